// Writes the binary cache of a text edge-list file (the reference's input format): every command
// line of this package accepts the cache in place of the text file and loads it without parsing.
//   cache_graph INPUT_FILE CACHE_FILE
#include <iostream>

#include "cli_common.h"

int main(int argc, char *argv[]) {
    if (argc != 3) {
        std::cout << "Usage: cache_graph INPUT_FILE CACHE_FILE" << std::endl;
        return 1;
    }
    const int st = cac_cache_convert(argv[1], argv[2]);
    if (st) return cli_fail("cac_cache_convert", st);
    uint32_t n = 0;
    uint64_t m = 0;
    cac_parse_header(argv[2], &n, &m);
    std::cout << argv[2] << "," << n << "," << m << std::endl;
    return 0;
}

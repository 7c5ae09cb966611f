// Harness (test infrastructure only) around the reference's comincut::number_of_trials
// (src/karger-stein/co_mincut.cpp:44-73): prints "n p trials" for each vertex count on the
// command line at the success probability given first.
#include <cstdio>
#include <cstdlib>

#include "co_mincut.h"

int main(int argc, char *argv[]) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: ks_trials PROBABILITY N...\n");
        return 1;
    }
    const double p = std::atof(argv[1]);
    for (int i = 2; i < argc; i++) {
        const int n = std::atoi(argv[i]);
        std::printf("%d %.17g %d\n", n, p, comincut::number_of_trials(n, p));
    }
    return 0;
}

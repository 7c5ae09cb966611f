/*
 * Stand-in for Boost's <boost/pending/disjoint_sets.hpp>, used ONLY to compile the
 * unmodified reference sources into oracle/_ref/ (test infrastructure).
 *
 * Implements the documented interface the reference calls
 * (src/DisjointSets.hpp:11,35,40; src/recursive-contract/disjoint_sets.hpp:8):
 *   disjoint_sets<RankPtr, ParentPtr>(rank, parent), find_set(x), link(x, y), union_set(x, y)
 * with the documented algorithm: union by rank plus full path compression. link(x, y)
 * first resolves both arguments to their representatives; the representative of larger
 * rank becomes the parent; on equal rank the second argument's representative becomes the
 * parent and its rank grows by one. Written from the interface documentation; no Boost
 * source is vendored or copied.
 */
#ifndef CAC_ORACLE_DISJOINT_SETS_STANDIN_HPP
#define CAC_ORACLE_DISJOINT_SETS_STANDIN_HPP

namespace boost {

template <class RankPtr, class ParentPtr>
class disjoint_sets {
    RankPtr rank_;
    ParentPtr parent_;

public:
    disjoint_sets(RankPtr r, ParentPtr p) : rank_(r), parent_(p) {}

    template <class Element>
    Element find_set(Element x) {
        Element root = x;
        while (parent_[root] != root) root = parent_[root];
        while (parent_[x] != root) {  // full path compression
            Element next = parent_[x];
            parent_[x] = root;
            x = next;
        }
        return root;
    }

    template <class Element>
    void link(Element x, Element y) {
        Element a = find_set(x), b = find_set(y);
        if (a == b) return;
        if (rank_[a] > rank_[b]) {
            parent_[b] = a;
        } else {
            parent_[a] = b;
            if (rank_[a] == rank_[b]) rank_[b] = rank_[b] + 1;
        }
    }

    template <class Element>
    void union_set(Element x, Element y) { link(x, y); }
};

}  // namespace boost

#endif

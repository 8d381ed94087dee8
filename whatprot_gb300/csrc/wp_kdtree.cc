// wp_kdtree.cc -- the kNN classifier's kd-tree, built on the host.
//
// NNClassifier keeps its training entries in a KDTree (kd-tree/kd-tree.h:
// 36-64) whose construction permutes the entries in place
// (kd-tree/make-node.h:28-80, kd-tree/max-min-nth.h:20-116).  The reference's
// k-hit set depends on the order in which the tree's search meets the
// entries and breaks equal distances by the entries' addresses in the
// permuted vector, so the device search (wp_kbest.cu) needs this exact
// permutation and these exact split values.  The build below takes the same
// decisions on the same FP64 coordinates:
//
//   * split dimension: the first one of largest (max - min), the maximum
//     starting from DBL_MIN and the minimum from DBL_MAX as the reference's
//     do;
//   * split position: the element the reference's own nth_element (not
//     std::nth_element) leaves at the middle, with its partition scans and
//     its handling of values equal to the pivot;
//   * a leaf when either side would hold fewer than k entries;
//   * split value (max_left + min_right) / 2.
//
// The permutation is kept as an index array, with the split dimension's
// values copied next to it for the partition scans.
#include <float.h>

#include <utility>
#include <vector>

#include "wp_kdtree.h"

namespace {

struct Builder {
    const double* X;  // [N][D], entries in input order
    int D;
    int k;
    std::vector<int> pos;    // tree position -> input index
    std::vector<double> v;   // the current split dimension's value at each position
    std::vector<KDNode>* nodes;
    int depth_max = 0;

    void swap_at(long i, long j) {
        std::swap(pos[i], pos[j]);
        std::swap(v[i], v[j]);
    }

    // One pass of the reference's partition around the value at `pivot`:
    // the pivot is parked at the end, the left scan stops at a larger value
    // and swaps it to the right cursor, the right scan stops at a value not
    // larger and swaps it to the left cursor; values equal to the pivot's are
    // counted as the scans pass them.  Returns the final left cursor.
    long split_pass(long begin, long end, long pivot, int* equal) {
        *equal = 0;
        long l = begin, r = end - 1;
        const double pv = v[pivot];
        swap_at(pivot, r);
        while (l < r) {
            for (; l < r; l++) {
                if (v[l] == pv) ++*equal;
                if (v[l] > pv) {
                    swap_at(l, r--);
                    break;
                }
            }
            for (; l < r; r--) {
                if (v[r] == pv) ++*equal;
                if (v[r] <= pv) {
                    swap_at(r, l++);
                    break;
                }
            }
        }
        return l;
    }

    // The second partition the reference runs when the middle falls among
    // values equal to the pivot: around the value at end - 1, values below
    // it to the left.
    void split_below(long begin, long end) {
        long l = begin, r = end - 1;
        const double pv = v[r];
        while (l < r) {
            for (; l < r; l++)
                if (v[l] >= pv) {
                    swap_at(l, r--);
                    break;
                }
            for (; l < r; r--)
                if (v[r] < pv) {
                    swap_at(r, l++);
                    break;
                }
        }
    }

    // The position the reference's nth_element returns for `nth` in
    // [begin, end): everything left of it strictly below everything from
    // it on.
    long middle(long begin, long end, long nth) {
        for (;;) {
            int equal = 0;
            const long hi = split_pass(begin, end, nth, &equal);
            const long lo = hi - equal;
            if (lo <= nth && nth <= hi) {
                if (nth - lo > hi - nth) return hi + 1;
                split_below(begin, hi + 1);
                return lo;
            }
            if (nth < lo) {
                split_below(begin, hi + 1);
                end = lo;
            } else {
                begin = hi + 1;
            }
        }
    }

    int make(long begin, long end, int depth) {
        if (depth > depth_max) depth_max = depth;
        double lo[64], hi[64];
        for (int i = 0; i < D; i++) {
            lo[i] = DBL_MAX;
            hi[i] = DBL_MIN;
        }
        for (long e = begin; e < end; e++) {
            const double* row = X + (long)pos[e] * D;
            for (int i = 0; i < D; i++) {
                if (row[i] < lo[i]) lo[i] = row[i];
                if (hi[i] < row[i]) hi[i] = row[i];
            }
        }
        int s = -1;
        double widest = -1.0;
        for (int i = 0; i < D; i++)
            if (hi[i] - lo[i] > widest) {
                widest = hi[i] - lo[i];
                s = i;
            }
        for (long e = begin; e < end; e++) v[e] = X[(long)pos[e] * D + s];
        const long nth = middle(begin, end, begin + (end - begin) / 2);
        const int id = (int)nodes->size();
        nodes->push_back(KDNode());
        if (nth - begin < k || end - nth < k) {
            KDNode& n = (*nodes)[id];
            n.leaf = 1;
            n.begin = (int)begin;
            n.end = (int)end;
            return id;
        }
        double max_left = DBL_MIN, min_right = DBL_MAX;
        for (long e = begin; e < nth; e++)
            if (max_left < v[e]) max_left = v[e];
        for (long e = nth; e < end; e++)
            if (v[e] < min_right) min_right = v[e];
        const int left = make(begin, nth, depth + 1);
        const int right = make(nth, end, depth + 1);
        KDNode& n = (*nodes)[id];
        n.s = s;
        n.left = left;
        n.right = right;
        n.max_left = max_left;
        n.min_right = min_right;
        n.split = (max_left + min_right) / 2;
        return id;
    }
};

}  // namespace

int wp_kdtree_build(const double* coords, int N, int D, int k, std::vector<int>* perm,
                    std::vector<KDNode>* nodes, int* max_depth) {
    nodes->clear();
    perm->clear();
    *max_depth = 0;
    if (D < 1 || D > 64 || N < 0) return -1;
    if (N == 0) return 0;
    Builder b;
    b.X = coords;
    b.D = D;
    b.k = k;
    b.pos.resize(N);
    for (int i = 0; i < N; i++) b.pos[i] = i;
    b.v.assign(N, 0.0);
    b.nodes = nodes;
    b.make(0, N, 0);
    *max_depth = b.depth_max;
    perm->swap(b.pos);
    return 0;
}

// wp_kdtree.h -- the kNN classifier's kd-tree (host build, device search).
#pragma once

#include <vector>

// One node of the tree as make_node creates it (kd-tree/make-node.h:28-80,
// internal-node.h:28-37, leaf-node.h:22-24).  The device search reads the
// same struct.
struct KDNode {
    double split = 0.0;      // (max_left + min_right) / 2
    double max_left = 0.0;   // largest split-dimension value on the left
    double min_right = 0.0;  // smallest on the right
    int s = 0;               // split dimension
    int left = -1, right = -1;
    int begin = 0, end = 0;  // a leaf's tree positions [begin, end)
    int leaf = 0;
    int pad = 0;
};

// Builds the tree of N entries with coordinates coords [N][D] (input order,
// D <= 64) for k: perm[i] is the input index of the entry at tree position
// i, nodes[0] is the root, max_depth the deepest level (root 0).  Returns 0,
// or -1 for a shape it does not take.
int wp_kdtree_build(const double* coords, int N, int D, int k, std::vector<int>* perm,
                    std::vector<KDNode>* nodes, int* max_depth);

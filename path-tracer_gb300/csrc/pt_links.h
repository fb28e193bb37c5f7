// pt_links.h - parent links of a binary BVH (host side), used by the
// precision form to break exact-t ties in the reference's traversal order.
#pragma once

#include <stdint.h>

#include <vector>

#include "../../include/pt.h"
#include "../../include/pt_precision.h"

namespace ptw {

// parent[i]: parent of binary node i (root: 0xffffffff); leaf_of[t]: the leaf
// holding triangle t.  False if a child or triangle range is out of bounds.
bool build_bvh_links(const pt_bvh_node* nodes, uint64_t node_count, uint64_t tri_count, uint32_t* parent,
                     uint32_t* leaf_of);

// pt_build_wide_bvh in one pass, into a vector sized by the build
int build_wide_bvh(const pt_bvh_node* nodes, uint64_t node_count, uint32_t max_leaf_triangles,
                   std::vector<pt_wide_node>& wide, uint32_t* wide_depth);

}  // namespace ptw

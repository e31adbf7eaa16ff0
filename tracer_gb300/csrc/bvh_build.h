// bvh_build.h -- host builder of the reference's BVH (see bvh_build.cpp).
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "../../include/tracer_gpu.h"
#include "tr_math.cuh"

namespace trg {

struct BvhResult {
  std::vector<tr_bvh_node32> nodes;  // reference LinearBVHNode layout, depth-first
  std::vector<uint32_t> order;       // leaf slot -> primitive index
  int depth = 0;                     // deepest node level (root = 0)
};

// lo/hi: 3 floats per primitive (world bounds in primitive-list order).
BvhResult build_reference_bvh(const float* lo, const float* hi, size_t n, int max_leaf_prims);

}  // namespace trg

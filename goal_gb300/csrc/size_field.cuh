// Isotropic target size field (get_iso_target_size, src/goal_size_field.cpp:139-151).
#pragma once

#include "disc.cuh"

namespace goal {

// err: per-element error indicators on the device, in the caller's element
// order; vtx_size: per-node target sizes on the device.
void iso_target_size(const Disc& d, const double* err, int target, double* vtx_size, cudaStream_t st);

}  // namespace goal

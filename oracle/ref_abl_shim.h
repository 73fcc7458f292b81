/*
 * ref_abl_shim.h -- stand-ins that let the ablation scans and the
 * non-interleaved WPK1 kernel of the reference's optimization.cu (lines
 * 91-114 and 144-442 of thejonwong/warpkernel) compile with g++ and run on the
 * CPU.  TEST INFRASTRUCTURE ONLY (builds oracle/_ref/libwkref_abl.so, see
 * Makefile).  The compiled lines use std::vector, WARP_SIZE, `uint`, CUDA
 * kernel qualifiers, the thread-index built-ins and fetch_cache (a texture
 * fetch in the reference; a plain read here, the cache = false form).
 */
#pragma once
#include <sys/types.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>

#define WARP_SIZE 32
#define __device__
#define __global__
#define __inline__ inline

struct emu_dim3 {
  unsigned x, y, z;
};
extern emu_dim3 threadIdx, blockIdx, blockDim;

template <bool usecache>
inline double fetch_cache(const int &i, const double *x) {
  return x[i];
}

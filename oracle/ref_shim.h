/*
 * ref_shim.h -- stand-ins that let the reference's host scan and WPK1 kernels
 * (warpkernel.hpp lines 27-771 of thejonwong/warpkernel) compile with g++ and
 * run on the CPU.  TEST INFRASTRUCTURE ONLY (builds oracle/_ref/, see Makefile).
 *
 * The reference needs CUSP (absent), texture references (removed from CUDA)
 * and CUDA launch syntax (only in the engine class, which is not compiled).
 * The stand-ins below provide just the names the compiled lines use:
 *   - cusp::array1d / csr_matrix as host vectors (device arrays live on the
 *     host here, so process() can be read back directly);
 *   - a do-nothing texture type (kernels are run with cache = false);
 *   - threadIdx / blockIdx / blockDim as globals set by the CPU emulator.
 */
#pragma once
#include <sys/types.h>

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <limits>
#include <string>
#include <utility>
#include <vector>

#define WARP_SIZE 32
#define __device__
#define __global__
#define __inline__ inline
#define __shared__

struct int2 {
  int x, y;
};
enum cudaTextureReadMode { cudaReadModeElementType };
template <class T, int Dim, int Mode>
struct texture {};
template <class T, int Dim, int Mode>
inline int2 tex1Dfetch(const texture<T, Dim, Mode> &, int) {
  return int2{0, 0};
}
inline double __hiloint2double(int hi, int lo) {
  unsigned long long b = ((unsigned long long)(unsigned)hi << 32) | (unsigned)lo;
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
}

struct emu_dim3 {
  unsigned x, y, z;
};
extern emu_dim3 threadIdx, blockIdx, blockDim;

namespace cusp {
struct device_memory {};
struct host_memory {};
template <class T, class Space>
struct array1d : std::vector<T> {
  using std::vector<T>::vector;
  array1d() {}
  template <class S2>
  array1d(const array1d<T, S2> &o) : std::vector<T>(o) {}
  template <class S2>
  array1d &operator=(const array1d<T, S2> &o) {
    std::vector<T>::operator=(o);
    return *this;
  }
  array1d &operator=(const std::vector<T> &o) {
    std::vector<T>::operator=(o);
    return *this;
  }
};
template <class I, class V, class Space>
struct csr_matrix {
  array1d<I, Space> row_offsets, column_indices;
  array1d<V, Space> values;
};
namespace system {
namespace cuda {}
}  // namespace system
}  // namespace cusp

namespace thrust {
template <class T>
T *raw_pointer_cast(T *p) {
  return p;
}
template <class A, class B, class C>
void scatter(A, A, B, C) {}
}  // namespace thrust

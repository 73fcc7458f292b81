// wk_fegen.cu -- finite-element test matrices and vectors generated on the
// device, plus element-type conversion.  Not part of the reference's API: the
// reference drivers read user Matrix Market files; these kernels produce the
// synthetic matrices of the benchmark configurations directly in HBM.
//
// Numbering and arithmetic are shared with the CPU generator used by the tests
// (same counter-based hash, same floating-point operations in the same order),
// so both give bit-identical matrices.
#include <cuda_bf16.h>

#include "wk_internal.cuh"

namespace wk {
namespace {

// splitmix64 finaliser (Steele, Lea, Flood 2014).
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ULL;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return z;
}
__host__ __device__ __forceinline__ uint64_t stream_base(uint64_t seed, uint64_t tag) {
  return mix64(seed * 0x9E3779B97F4A7C15ULL + tag);
}
__device__ __forceinline__ uint64_t hkey(uint64_t base, uint64_t key) {
  return mix64(base ^ (key * 0xD1B54A32D192ED03ULL));
}
__device__ __forceinline__ double unit_open(uint64_t h) {
  return ((double)(h >> 12) + 0.5) * 0x1.0p-52;
}
__device__ __forceinline__ double gauss4(uint64_t base, uint64_t key) {
  double s = unit_open(hkey(base, key * 4 + 0));
  s = s + unit_open(hkey(base, key * 4 + 1));
  s = s + unit_open(hkey(base, key * 4 + 2));
  s = s + unit_open(hkey(base, key * 4 + 3));
  return (s - 2.0) * 1.7320508075688772;
}

enum { TAG_STENCIL = 1, TAG_ELEMENT = 2, TAG_VECTOR = 16 };

struct Mesh {
  int dim, ex, ey, ez, dof;
  int64_t nx, ny, nzn;
  int npe, nb;
};

__host__ __device__ __forceinline__ int64_t axis_count(int64_t i, int64_t n) {
  return (i > 0) + 1 + (i + 1 < n);
}
// sum of axis_count over k < i
__device__ __forceinline__ int64_t axis_prefix(int64_t i, int64_t n) {
  if (i == 0) return 0;
  if (n == 1) return 1;
  if (i >= n) return 3 * n - 2;
  return 2 + 3 * (i - 1);
}

// Row pointers in closed form: node-major, `dof` rows per node.
__global__ void k_fe_rowptr(Mesh m, int32_t *__restrict__ rowptr, int64_t nrows) {
  const int64_t Tx = axis_prefix(m.nx, m.nx), Ty = axis_prefix(m.ny, m.ny);
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    if (r == nrows) {
      rowptr[r] = (int32_t)(Tx * Ty * axis_prefix(m.nzn, m.nzn) * m.dof * m.dof);
      continue;
    }
    int64_t n = r / m.dof, c = r % m.dof;
    int64_t ix = n % m.nx, iy = (n / m.nx) % m.ny, iz = n / (m.nx * m.ny);
    int64_t cx = axis_count(ix, m.nx), cy = axis_count(iy, m.ny), cz = axis_count(iz, m.nzn);
    int64_t before = Tx * Ty * axis_prefix(iz, m.nzn) + cz * Tx * axis_prefix(iy, m.ny) +
                     cz * cy * axis_prefix(ix, m.nx);
    rowptr[r] = (int32_t)(before * m.dof * m.dof + c * cx * cy * cz * m.dof);
  }
}

// Element blocks K_e = G G^T / nb + 0.01 I, times the element volume.
// One block per element; G staged in shared memory.
__global__ void k_fe_element(Mesh m, uint64_t base, double vol, int64_t nelem, double *__restrict__ K) {
  extern __shared__ double G[];
  const int nb = m.nb;
  for (int64_t e = blockIdx.x; e < nelem; e += gridDim.x) {
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x)
      G[t] = gauss4(base, ((uint64_t)e * nb + t / nb) * nb + t % nb);
    __syncthreads();
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
      int a = t / nb, b = t % nb;
      double acc = 0.0;
      for (int q = 0; q < nb; q++) acc = fma(G[a * nb + q], G[b * nb + q], acc);
      double k = acc / (double)nb;
      if (a == b) k = k + 0.01;
      K[(size_t)e * nb * nb + t] = k * vol;
    }
    __syncthreads();
  }
}

// Columns and values of each row (one thread per row).
__global__ void k_fe_rows(Mesh m, int value_mode, uint64_t base, const int32_t *__restrict__ rowptr,
                          int64_t nrows, const double *__restrict__ K, int32_t *__restrict__ cols,
                          double *__restrict__ vals) {
  const uint64_t N = (uint64_t)nrows;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t n = r / m.dof;
    const int c = (int)(r % m.dof);
    const int64_t ix = n % m.nx, iy = (n / m.nx) % m.ny, iz = n / (m.nx * m.ny);
    int64_t k = rowptr[r];
    double diag_sum = 0.0;
    int64_t diag_k = -1;
    for (int dz = -1; dz <= 1; dz++) {
      const int64_t jz = iz + dz;
      if (jz < 0 || jz >= m.nzn) continue;
      for (int dy = -1; dy <= 1; dy++) {
        const int64_t jy = iy + dy;
        if (jy < 0 || jy >= m.ny) continue;
        for (int dx = -1; dx <= 1; dx++) {
          const int64_t jx = ix + dx;
          if (jx < 0 || jx >= m.nx) continue;
          const int64_t nj = jx + m.nx * (jy + m.ny * jz);
          for (int c2 = 0; c2 < m.dof; c2++, k++) {
            const int64_t j = nj * m.dof + c2;
            if (cols) cols[k] = (int32_t)j;
            if (!vals) continue;
            if (value_mode == 0) {
              if (j == r) {
                diag_k = k;
                continue;
              }
              uint64_t lo = (uint64_t)(j < r ? j : r), hi = (uint64_t)(j < r ? r : j);
              double v = -unit_open(hkey(base, lo * N + hi));
              vals[k] = v;
              diag_sum = diag_sum + fabs(v);
            } else {
              double s = 0.0;
              const int64_t z0 = (iz > jz ? iz : jz) - 1, z1 = iz < jz ? iz : jz;
              const int64_t y0 = (iy > jy ? iy : jy) - 1, y1 = iy < jy ? iy : jy;
              const int64_t x0 = (ix > jx ? ix : jx) - 1, x1 = ix < jx ? ix : jx;
              for (int64_t ez_ = z0; ez_ <= z1; ez_++) {
                if (ez_ < 0 || ez_ >= m.ez) continue;
                if (m.dim == 2 && ez_ != 0) continue;
                for (int64_t ey_ = y0; ey_ <= y1; ey_++) {
                  if (ey_ < 0 || ey_ >= m.ey) continue;
                  for (int64_t ex_ = x0; ex_ <= x1; ex_++) {
                    if (ex_ < 0 || ex_ >= m.ex) continue;
                    int li = (int)(ix - ex_) + 2 * (int)(iy - ey_);
                    int lj = (int)(jx - ex_) + 2 * (int)(jy - ey_);
                    if (m.dim == 3) {
                      li += 4 * (int)(iz - ez_);
                      lj += 4 * (int)(jz - ez_);
                    }
                    const int64_t e = ex_ + (int64_t)m.ex * (ey_ + (int64_t)m.ey * ez_);
                    s = s + K[(size_t)e * m.nb * m.nb + (size_t)(li * m.dof + c) * m.nb + lj * m.dof + c2];
                  }
                }
              }
              vals[k] = s;
            }
          }
        }
      }
    }
    if (vals && value_mode == 0) vals[diag_k] = 1.01 * diag_sum;
  }
}

__global__ void k_uniform(uint64_t base, double *__restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = 2.0 * unit_open(hkey(base, (uint64_t)i)) - 1.0;
}

__device__ __forceinline__ double to_f64(const void *p, int dt, int64_t i) {
  switch (dt) {
    case WK_F64: return ((const double *)p)[i];
    case WK_F32: return (double)((const float *)p)[i];
    default: return (double)__bfloat162float(((const __nv_bfloat16 *)p)[i]);
  }
}

__global__ void k_convert(const void *src, int sdt, void *dst, int ddt, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (sdt == WK_F32 && ddt == WK_BF16) {
      ((__nv_bfloat16 *)dst)[i] = __float2bfloat16_rn(((const float *)src)[i]);
      continue;
    }
    double v = to_f64(src, sdt, i);
    switch (ddt) {
      case WK_F64: ((double *)dst)[i] = v; break;
      case WK_F32: ((float *)dst)[i] = __double2float_rn(v); break;
      default: ((__nv_bfloat16 *)dst)[i] = __double2bfloat16(v); break;
    }
  }
}

unsigned grid_for(int64_t n, int bs) {
  int64_t g = (n + bs - 1) / bs;
  if (g < 1) g = 1;
  if (g > 152 * 64) g = 152 * 64;
  return (unsigned)g;
}

}  // namespace

wk_status launch_fe_fill(int dim, int ex, int ey, int ez, int dof, int value_mode, uint64_t seed, int32_t *rowptr,
                         int32_t *cols, double *vals, cudaStream_t st) {
  Mesh m;
  m.dim = dim; m.ex = ex; m.ey = ey; m.ez = dim == 3 ? ez : 1; m.dof = dof;
  m.nx = ex + 1; m.ny = ey + 1; m.nzn = dim == 3 ? ez + 1 : 1;
  m.npe = dim == 3 ? 8 : 4;
  m.nb = m.npe * dof;
  const int64_t nrows = m.nx * m.ny * m.nzn * dof;
  DevBuf rp_tmp;
  int32_t *rp = rowptr;
  if (!rp) {
    if (!cols && !vals) return WK_OK;
    WK_TRY(rp_tmp.alloc((size_t)(nrows + 1) * 4));
    rp = rp_tmp.as<int32_t>();
  }
  k_fe_rowptr<<<grid_for(nrows + 1, 256), 256, 0, st>>>(m, rp, nrows);
  WK_CHECK_LAUNCH();
  DevBuf K;
  uint64_t base = 0;
  if (vals && value_mode == 1) {
    const int64_t nelem = (int64_t)m.ex * m.ey * m.ez;
    WK_TRY(K.alloc((size_t)nelem * m.nb * m.nb * 8));
    const double h = 1.0 / (double)ex;
    const double vol = dim == 3 ? h * h * h : h * h;
    base = stream_base(seed, TAG_ELEMENT);
    unsigned g = (unsigned)(nelem < 152 * 256 ? nelem : 152 * 256);
    k_fe_element<<<g, 256, (size_t)m.nb * m.nb * 8, st>>>(m, base, vol, nelem, K.as<double>());
    WK_CHECK_LAUNCH();
  } else if (vals) {
    base = stream_base(seed, TAG_STENCIL);
  }
  if (cols || vals) {
    k_fe_rows<<<grid_for(nrows, 128), 128, 0, st>>>(m, value_mode, base, rp, nrows, K.as<double>(), cols, vals);
    WK_CHECK_LAUNCH();
  }
  WK_CUDA(cudaStreamSynchronize(st));  // temporaries are freed on return
  return WK_OK;
}

wk_status launch_uniform(uint64_t seed, uint64_t stream_id, double *x, int64_t n, cudaStream_t st) {
  if (!n) return WK_OK;
  k_uniform<<<grid_for(n, 256), 256, 0, st>>>(stream_base(seed, TAG_VECTOR + stream_id), x, n);
  WK_CHECK_LAUNCH();
  return WK_OK;
}

wk_status launch_convert(const void *src, int sdt, void *dst, int ddt, int64_t n, cudaStream_t st) {
  if (!n) return WK_OK;
  k_convert<<<grid_for(n, 256), 256, 0, st>>>(src, sdt, dst, ddt, n);
  WK_CHECK_LAUNCH();
  return WK_OK;
}

}  // namespace wk

/*
 * wk_fegen.c -- CPU finite-element test-matrix generator.
 *
 * TEST INFRASTRUCTURE ONLY.  A restatement, for the CPU, of the product's
 * device generator (warpkernel_gb300/csrc/fegen.cu): same mesh numbering, same
 * counter-based hash, same floating-point operations in the same order, so
 * both produce bit-identical CSR matrices.  Used by the CPU tests and by the
 * CPU arms of bench.py, which must not touch the GPU library.
 *
 * Mesh: dim 2 = ex x ey Q1 quads, dim 3 = ex x ey x ez trilinear hexes,
 * `dof` unknowns per node.  Node id = ix + nx*(iy + ny*iz), row = dof*node + c.
 * Row pattern: every dof of every node sharing an element with the row's node,
 * columns ascending.
 */
#include "wk_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* splitmix64 finaliser (Steele, Lea, Flood 2014). */
static inline uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ULL;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return z;
}
static inline uint64_t stream_base(uint64_t seed, uint64_t tag) {
  return mix64(seed * 0x9E3779B97F4A7C15ULL + tag);
}
static inline uint64_t hkey(uint64_t base, uint64_t key) {
  return mix64(base ^ (key * 0xD1B54A32D192ED03ULL));
}
/* (0,1), exactly representable: ((h >> 12) + 0.5) * 2^-52 */
static inline double unit_open(uint64_t h) {
  return ((double)(h >> 12) + 0.5) * 0x1.0p-52;
}
/* approximately N(0,1): Irwin-Hall sum of four uniforms, unit variance */
static inline double gauss4(uint64_t base, uint64_t key) {
  double s = unit_open(hkey(base, key * 4 + 0));
  s = s + unit_open(hkey(base, key * 4 + 1));
  s = s + unit_open(hkey(base, key * 4 + 2));
  s = s + unit_open(hkey(base, key * 4 + 3));
  return (s - 2.0) * 1.7320508075688772;
}

enum { TAG_STENCIL = 1, TAG_ELEMENT = 2, TAG_VECTOR = 16 };

typedef struct {
  int dim, ex, ey, ez, dof;
  int64_t nx, ny, nzn; /* nodes per axis (nzn = 1 in 2-D) */
  int npe, nb;         /* nodes per element, block size */
} mesh_t;

static int mesh_init(mesh_t *m, int dim, int ex, int ey, int ez, int dof) {
  if ((dim != 2 && dim != 3) || ex < 1 || ey < 1 || dof < 1 || (dim == 3 && ez < 1)) return 1;
  m->dim = dim; m->ex = ex; m->ey = ey; m->ez = dim == 3 ? ez : 1; m->dof = dof;
  m->nx = ex + 1; m->ny = ey + 1; m->nzn = dim == 3 ? ez + 1 : 1;
  m->npe = dim == 3 ? 8 : 4;
  m->nb = m->npe * dof;
  return 0;
}

static inline int axis_count(int64_t i, int64_t n) { return (i > 0) + 1 + (i + 1 < n); }

int wko_fe_size(int dim, int ex, int ey, int ez, int dof, int64_t *nrows, int64_t *nnz) {
  mesh_t m;
  if (mesh_init(&m, dim, ex, ey, ez, dof)) return 1;
  int64_t nn = m.nx * m.ny * m.nzn;
  /* sum over nodes of the neighbour count factorises per axis */
  int64_t sx = 0, sy = 0, sz = 0;
  for (int64_t i = 0; i < m.nx; i++) sx += axis_count(i, m.nx);
  for (int64_t i = 0; i < m.ny; i++) sy += axis_count(i, m.ny);
  for (int64_t i = 0; i < m.nzn; i++) sz += axis_count(i, m.nzn);
  *nrows = nn * dof;
  *nnz = sx * sy * sz * (int64_t)dof * dof;
  return 0;
}

/* Element stiffness entry K_e[a][b] = (sum_m G[a][m] G[b][m]) / nb + 0.01 [a==b],
 * times the element volume h^dim with h = 1/ex. */
static double element_entry(const double *G, int nb, int a, int b, double vol) {
  double acc = 0.0;
  for (int q = 0; q < nb; q++) acc = fma(G[a * nb + q], G[b * nb + q], acc);
  double k = acc / (double)nb;
  if (a == b) k = k + 0.01;
  return k * vol;
}

static void element_G(uint64_t base, int64_t e, int nb, double *G) {
  for (int a = 0; a < nb; a++)
    for (int q = 0; q < nb; q++) G[a * nb + q] = gauss4(base, ((uint64_t)e * nb + a) * nb + q);
}

int wko_fe_fill(int dim, int ex, int ey, int ez, int dof, int value_mode, uint64_t seed,
                int32_t *rowptr, int32_t *cols, double *vals, int nthreads) {
  mesh_t m;
  if (mesh_init(&m, dim, ex, ey, ez, dof)) return 1;
  int64_t nrows, nnz;
  wko_fe_size(dim, ex, ey, ez, dof, &nrows, &nnz);
  if (nnz > 2147483647LL) return 2;
  if (nthreads <= 0) nthreads = wko_max_threads();
  const int64_t nn = m.nx * m.ny * m.nzn;

  /* row pointers: rows of one node share a length */
  int32_t *rp = rowptr;
  int32_t *tmp = NULL;
  if (!rp) {
    tmp = (int32_t *)malloc((size_t)(nrows + 1) * sizeof(int32_t));
    if (!tmp) return 3;
    rp = tmp;
  }
  {
    int64_t acc = 0;
    rp[0] = 0;
    for (int64_t n = 0; n < nn; n++) {
      int64_t ix = n % m.nx, iy = (n / m.nx) % m.ny, iz = n / (m.nx * m.ny);
      int64_t len = (int64_t)axis_count(ix, m.nx) * axis_count(iy, m.ny) * axis_count(iz, m.nzn) * dof;
      for (int c = 0; c < dof; c++) {
        acc += len;
        rp[n * dof + c + 1] = (int32_t)acc;
      }
    }
  }
  if (cols) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t n = 0; n < nn; n++) {
      int64_t ix = n % m.nx, iy = (n / m.nx) % m.ny, iz = n / (m.nx * m.ny);
      for (int c = 0; c < dof; c++) {
        int64_t k = rp[n * dof + c];
        for (int dz = -1; dz <= 1; dz++) {
          int64_t jz = iz + dz;
          if (jz < 0 || jz >= m.nzn) continue;
          for (int dy = -1; dy <= 1; dy++) {
            int64_t jy = iy + dy;
            if (jy < 0 || jy >= m.ny) continue;
            for (int dx = -1; dx <= 1; dx++) {
              int64_t jx = ix + dx;
              if (jx < 0 || jx >= m.nx) continue;
              int64_t nj = jx + m.nx * (jy + m.ny * jz);
              for (int c2 = 0; c2 < dof; c2++) cols[k++] = (int32_t)(nj * dof + c2);
            }
          }
        }
      }
    }
  }
  if (vals && value_mode == 0) {
    const uint64_t base = stream_base(seed, TAG_STENCIL);
    const uint64_t N = (uint64_t)nrows;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t r = 0; r < nrows; r++) {
      /* columns are needed for the values: recompute them if not requested */
      int64_t n = r / dof;
      int64_t ix = n % m.nx, iy = (n / m.nx) % m.ny, iz = n / (m.nx * m.ny);
      int64_t k0 = rp[r];
      double diag_sum = 0.0;
      int64_t diag_k = -1, k = k0;
      for (int dz = -1; dz <= 1; dz++) {
        int64_t jz = iz + dz;
        if (jz < 0 || jz >= m.nzn) continue;
        for (int dy = -1; dy <= 1; dy++) {
          int64_t jy = iy + dy;
          if (jy < 0 || jy >= m.ny) continue;
          for (int dx = -1; dx <= 1; dx++) {
            int64_t jx = ix + dx;
            if (jx < 0 || jx >= m.nx) continue;
            int64_t nj = jx + m.nx * (jy + m.ny * jz);
            for (int c2 = 0; c2 < dof; c2++, k++) {
              uint64_t j = (uint64_t)(nj * dof + c2);
              if ((int64_t)j == r) {
                diag_k = k;
                continue;
              }
              uint64_t lo = j < (uint64_t)r ? j : (uint64_t)r, hi = j < (uint64_t)r ? (uint64_t)r : j;
              double v = -unit_open(hkey(base, lo * N + hi));
              vals[k] = v;
              diag_sum = diag_sum + fabs(v);
            }
          }
        }
      }
      vals[diag_k] = 1.01 * diag_sum;
    }
  } else if (vals && value_mode == 1) {
    const uint64_t base = stream_base(seed, TAG_ELEMENT);
    const int nb = m.nb;
    const double h = 1.0 / (double)ex;
    const double vol = dim == 3 ? h * h * h : h * h;
    const int64_t epl = (int64_t)m.ex * m.ey; /* elements per z-plane */
    /* element stiffness blocks of two element planes (rolling) */
    double *Kp[2];
    Kp[0] = (double *)malloc((size_t)epl * nb * nb * sizeof(double));
    Kp[1] = (double *)malloc((size_t)epl * nb * nb * sizeof(double));
    if (!Kp[0] || !Kp[1]) {
      free(Kp[0]); free(Kp[1]); free(tmp);
      return 3;
    }
    const int64_t planes_e = m.ez; /* 1 in 2-D */
    for (int64_t kz = 0; kz < m.nzn; kz++) {
      /* element plane kz (if any) into Kp[kz & 1] */
      if (kz < planes_e) {
        double *K = Kp[kz & 1];
#pragma omp parallel num_threads(nthreads)
        {
          double *G = (double *)malloc((size_t)nb * nb * sizeof(double));
#pragma omp for schedule(static)
          for (int64_t el = 0; el < epl; el++) {
            int64_t e = kz * epl + el;
            element_G(base, e, nb, G);
            double *Ke = K + el * nb * nb;
            for (int a = 0; a < nb; a++)
              for (int b = 0; b < nb; b++) Ke[a * nb + b] = element_entry(G, nb, a, b, vol);
          }
          free(G);
        }
      }
      /* rows of node plane kz */
      int64_t n0 = kz * m.nx * m.ny, n1 = n0 + m.nx * m.ny;
#pragma omp parallel for schedule(static) num_threads(nthreads)
      for (int64_t n = n0; n < n1; n++) {
        int64_t ix = n % m.nx, iy = (n / m.nx) % m.ny, iz = kz;
        for (int c = 0; c < dof; c++) {
          int64_t k = rp[n * dof + c];
          for (int dz = -1; dz <= 1; dz++) {
            int64_t jz = iz + dz;
            if (jz < 0 || jz >= m.nzn) continue;
            for (int dy = -1; dy <= 1; dy++) {
              int64_t jy = iy + dy;
              if (jy < 0 || jy >= m.ny) continue;
              for (int dx = -1; dx <= 1; dx++) {
                int64_t jx = ix + dx;
                if (jx < 0 || jx >= m.nx) continue;
                for (int c2 = 0; c2 < dof; c2++, k++) {
                  double s = 0.0;
                  /* elements holding both nodes, ascending element id */
                  for (int64_t ez_ = (iz > jz ? iz : jz) - 1; ez_ <= (iz < jz ? iz : jz); ez_++) {
                    if (ez_ < 0 || ez_ >= planes_e) continue;
                    if (dim == 2 && ez_ != 0) continue;
                    for (int64_t ey_ = (iy > jy ? iy : jy) - 1; ey_ <= (iy < jy ? iy : jy); ey_++) {
                      if (ey_ < 0 || ey_ >= m.ey) continue;
                      for (int64_t ex_ = (ix > jx ? ix : jx) - 1; ex_ <= (ix < jx ? ix : jx); ex_++) {
                        if (ex_ < 0 || ex_ >= m.ex) continue;
                        int li = (int)(ix - ex_) + 2 * (int)(iy - ey_);
                        int lj = (int)(jx - ex_) + 2 * (int)(jy - ey_);
                        if (dim == 3) {
                          li += 4 * (int)(iz - ez_);
                          lj += 4 * (int)(jz - ez_);
                        }
                        const double *Ke = Kp[ez_ & 1] + (ey_ * m.ex + ex_) * nb * nb;
                        s = s + Ke[(li * dof + c) * nb + lj * dof + c2];
                      }
                    }
                  }
                  vals[k] = s;
                }
              }
            }
          }
        }
      }
    }
    free(Kp[0]);
    free(Kp[1]);
  }
  free(tmp);
  return 0;
}

void wko_uniform_vec(uint64_t seed, uint64_t stream, double *x, int64_t n) {
  const uint64_t base = stream_base(seed, TAG_VECTOR + stream);
  for (int64_t i = 0; i < n; i++) x[i] = 2.0 * unit_open(hkey(base, (uint64_t)i)) - 1.0;
}

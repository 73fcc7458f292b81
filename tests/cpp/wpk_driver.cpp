// wpk_driver.cpp -- host code in the shape of the reference's wpk1.cu and
// wpk2.cu drivers, compiled against include/warpkernel.hpp (the drop-in
// surface) and run by tests/test_gpu_cpp_driver.py.
//
// Matrix: a Matrix Market file read with warpkernel::read_matrix_market_file
// (the drivers' cusp::io::read_matrix_market_file), or a finite-element
// matrix from the library's generator.  Reference y: a host CSR product (the
// drivers use CUSP's CSR multiply).  After WPK1 and WPK2 it runs the rowsort
// variant of optimize2.cu:740-796, run_assembly and a layout file round trip.
//
//   wpk_driver dim ex ey ez dof [ntests]
//   wpk_driver --mm file.mtx [ntests]
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <sstream>
#include <vector>

#include "warpkernel.hpp"

#define ValueType double
#define IndexType int

using namespace warpkernel;

typedef csr_matrix<IndexType, ValueType> csr;

static csr make_matrix(int dim, int ex, int ey, int ez, int dof) {
  int64_t n = 0, z = 0;
  check(wk_fe_size(dim, ex, ey, ez, dof, &n, &z));
  device_array<int32_t> rp(n + 1), c(z);
  device_array<double> v(z);
  check(wk_fe_fill(dim, ex, ey, ez, dof, 1, 7, rp.data(), c.data(), v.data(), nullptr));
  csr A;
  A.row_offsets = rp.to_host();
  A.column_indices = c.to_host();
  A.values = v.to_host();
  A.num_rows = (uint)n;
  A.num_entries = (uint)z;
  return A;
}

static std::vector<ValueType> csr_multiply(const csr &A, const std::vector<ValueType> &x) {
  std::vector<ValueType> y(A.num_rows, 0.0);
  for (uint r = 0; r < A.num_rows; r++) {
    ValueType s = 0;
    for (int k = A.row_offsets[r]; k < A.row_offsets[r + 1]; k++) s += A.values[k] * x[A.column_indices[k]];
    y[r] = s;
  }
  return y;
}

int main(int argc, char **argv) {
  csr A;
  int ntests = 1;
  if (argc >= 3 && std::string(argv[1]) == "--mm") {
    read_matrix_market_file(A, argv[2]);
    std::printf("Finished Loading %s\n", argv[2]);
    ntests = argc > 3 ? atoi(argv[3]) : 1;
  } else if (argc >= 6) {
    const int dim = atoi(argv[1]), ex = atoi(argv[2]), ey = atoi(argv[3]), ez = atoi(argv[4]), dof = atoi(argv[5]);
    ntests = argc > 6 ? atoi(argv[6]) : 1;
    A = make_matrix(dim, ex, ey, ez, dof);
  } else {
    std::fprintf(stderr, "usage: %s dim ex ey ez dof [ntests] | --mm file.mtx [ntests]\n", argv[0]);
    return 2;
  }
  uint N = A.num_rows, M = A.num_rows, nz = A.num_entries;
  std::vector<ValueType> x(N);
  srand(1);
  for (auto &v : x) v = ((ValueType)(rand() % 100)) / 100. - 0.3;
  std::vector<ValueType> y = csr_multiply(A, x);
  stats stats_all, stats_n, stats_r, stats_rx;
  int failures = 0;

  // ---- warp kernel 1 (wpk1.cu:118-244) ----
  {
    device_array<ValueType> dx = x;
    structure kernel1;
    kernel1.scan(nz, M, &A.values[0], &A.row_offsets[0], &A.column_indices[0]);
    std::vector<IndexType> reorder_cols = A.column_indices;
    kernel1.reorder_columns_coalesced(reorder_cols);
    device_array<ValueType> dreordered_x;
    kernel1.reorder_x(x, dreordered_x);
    engine<ValueType, IndexType> eng(kernel1, &A.values[0], &A.column_indices[0]);
    for (int wpb = 1; wpb <= 16; wpb++) {
      uint nblocks = (kernel1.nwarps + wpb - 1) / wpb, blocksize = wpb * WARP_SIZE;
      std::ostringstream tag;
      tag << "warps/block = " << wpb;
      {
        profiler norm;
        device_array<ValueType> dy(N, 0);
        for (int t = 0; t < ntests; t++) norm.add(eng.run<true>(nblocks, blocksize, dx.data(), dy.data()));
        std::vector<ValueType> ycheck = dy;
        if (eng.verify(y, ycheck)) {
          stats_all.add(norm.avg(), tag.str());
          stats_n.add(norm.avg(), tag.str());
        } else {
          std::printf("WPK1 failed (%s)\n", tag.str().c_str());
          failures++;
        }
      }
      std::vector<IndexType> restore_col = eng.device_colinds;
      {
        profiler reordered;
        device_array<ValueType> dy(N, 0);
        eng.device_colinds = reorder_cols;
        for (int t = 0; t < ntests; t++)
          reordered.add(eng.run_x<true>(nblocks, blocksize, dreordered_x.data(), dy.data()));
        std::vector<ValueType> ycheck = dy;
        if (eng.verify_x(y, ycheck)) {
          stats_all.add(reordered.avg(), tag.str());
          stats_r.add(reordered.avg(), tag.str());
        } else {
          std::printf("WPK1_r failed (%s)\n", tag.str().c_str());
          failures++;
        }
        eng.device_colinds = restore_col;
      }
      {
        profiler rowmap;
        device_array<ValueType> dy(N, 0);
        eng.device_colinds = reorder_cols;
        for (int t = 0; t < ntests; t++)
          rowmap.add(eng.run<false>(nblocks, blocksize, dreordered_x.data(), dy.data()));
        std::vector<ValueType> ycheck = dy;
        if (eng.verify(y, ycheck)) {
          stats_all.add(rowmap.avg(), tag.str());
          stats_rx.add(rowmap.avg(), tag.str());
        } else {
          std::printf("WPK1_rx failed (%s)\n", tag.str().c_str());
          failures++;
        }
        eng.device_colinds = restore_col;
      }
    }
  }
  std::printf("Fastest WPK1 (all) = %e [s] (%s)\n", stats_all.Min(), stats_all.Min_str().c_str());

  // ---- warp kernel 2 (wpk2.cu:136-287) ----
  {
    device_array<ValueType> dx = x;
    structure2 kernel2;
    kernel2.scan(nz, N, &A.values[0], &A.row_offsets[0], &A.column_indices[0], (int)N);
    int max_nz = kernel2.max_nz, min_nz = kernel2.min_nz;
    // wpk2.cu:156 truncates (max - min) * 0.1 to int, which is 0 (an endless
    // sweep) when max - min < 10; step by at least 1
    int inc = std::max(1, (int)((max_nz - min_nz) * 0.1));
    for (int threshold = min_nz; threshold <= max_nz; threshold += inc) {
      kernel2.scan(nz, N, &A.values[0], &A.row_offsets[0], &A.column_indices[0], threshold);
      std::vector<IndexType> reorder_cols = A.column_indices;
      kernel2.reorder_columns_coalesced(reorder_cols);
      device_array<ValueType> dreordered_x;
      kernel2.reorder_x(x, dreordered_x);
      engine<ValueType, IndexType> eng(kernel2, &A.values[0], &A.column_indices[0]);
      for (int wpb = 2; wpb <= 16; wpb += 2) {
        uint nblocks = (kernel2.nwarps + wpb - 1) / wpb, blocksize = wpb * WARP_SIZE;
        device_array<ValueType> dy(N, 0.);
        eng.run<true>(nblocks, blocksize, dx.data(), dy.data());
        std::vector<ValueType> ycheck = dy;
        if (!eng.verify(y, ycheck)) {
          std::printf("WPK2 failed (threshold %d, wpb %d)\n", threshold, wpb);
          failures++;
        }
        std::vector<IndexType> restore_col = eng.device_colinds;
        eng.device_colinds = reorder_cols;
        device_array<ValueType> dy2(N, 0.);
        eng.run_x<true>(nblocks, blocksize, dreordered_x.data(), dy2.data());
        std::vector<ValueType> ycheck2 = dy2;
        if (!eng.verify_x(y, ycheck2)) {
          std::printf("WPK2_r failed (threshold %d, wpb %d)\n", threshold, wpb);
          failures++;
        }
        eng.device_colinds = restore_col;
      }
    }
  }
  // ---- rowsort variant (optimize2.cu:740-796), run_assembly, layout file ----
  {
    structure2 kernel1;
    kernel1.scan(nz, N, &A.values[0], &A.row_offsets[0], &A.column_indices[0], 4);
    uint nblocks = (kernel1.nwarps + 3) / 4, blocksize = 4 * WARP_SIZE;
    std::vector<IndexType> reorder_cols = A.column_indices;
    kernel1.reorder_columns_rowsort(reorder_cols, A.row_offsets);
    device_array<ValueType> dreordered_x;
    kernel1.reorder_x(x, dreordered_x);
    std::vector<ValueType> A_new_values(nz);
    for (uint i = 0; i < nz; i++) A_new_values[i] = A.values[kernel1.reorder_A_rows[i]];
    engine<ValueType, IndexType> eng(kernel1, &A_new_values[0], &reorder_cols[0]);
    device_array<ValueType> dy(N, 0);
    eng.run_x<true>(nblocks, blocksize, dreordered_x.data(), dy.data());
    std::vector<ValueType> ycheck = dy;
    if (!eng.verify_x(y, ycheck)) {
      std::printf("WPK2_rex_rowsort failed\n");
      failures++;
    }
    // process / reorder (warpkernel.hpp:533-548, 750-769) into caller device arrays
    {
      device_array<ValueType> dv;
      device_array<IndexType> dc, drm, dwo;
      device_array<uint> dmx, dtpr, drow;
      kernel1.process(&A_new_values[0], &reorder_cols[0], dv, dc, drm, dmx, dwo, dtpr, drow);
      if (dv.to_host() != eng.device_values.to_host() || dc.to_host() != eng.device_colinds.to_host() ||
          drm.to_host() != kernel1.row_map || dtpr.to_host() != kernel1.threads_per_row ||
          drow.to_host() != kernel1.row_offset_warp || dwo.to_host() != kernel1.warp_offsets) {
        std::printf("structure2::process differs from the engine's arrays\n");
        failures++;
      }
      device_array<ValueType> dv2;
      kernel1.reorder_values_coalesced(A_new_values, dv2);
      if (dv2.to_host() != dv.to_host()) {
        std::printf("reorder_values_coalesced differs\n");
        failures++;
      }
    }
    device_array<ValueType> vslots;
    kernel1.reorder_values_coalesced_rowsort(A.values, vslots);
    if (vslots.to_host() != eng.device_values.to_host()) {
      std::printf("reorder_values_coalesced_rowsort differs from the engine's values\n");
      failures++;
    }
    // run_assembly: row sums of the stored values
    std::vector<ValueType> rowsum(N, 0.0);
    for (uint r = 0; r < N; r++)
      for (int k = A.row_offsets[r]; k < A.row_offsets[r + 1]; k++) rowsum[r] += A.values[k];
    device_array<ValueType> ds(N, 0);
    eng.run_assembly<true>(nblocks, blocksize, ds.data());
    std::vector<ValueType> scheck = ds;
    if (!eng.verify(rowsum, scheck)) {
      std::printf("run_assembly failed\n");
      failures++;
    }
    // the layout survives a file round trip
    kernel1.save("wpk_layout.bin");
    structure2 loaded;
    loaded.load("wpk_layout.bin");
    if (loaded.row_map != kernel1.row_map || loaded.reorder_rows != kernel1.reorder_rows ||
        loaded.warp_offsets != kernel1.warp_offsets || loaded.threads_per_row != kernel1.threads_per_row ||
        loaded.row_offset_warp != kernel1.row_offset_warp || loaded.allocate_nz != kernel1.allocate_nz) {
      std::printf("layout file round trip differs\n");
      failures++;
    }
    std::remove("wpk_layout.bin");
  }
  // errors surface as exceptions, not exit(): a malformed CSR
  try {
    structure bad;
    std::vector<int> rp = {0, 3, 2};
    uint bnz = 2, bn = 2;
    bad.scan(bnz, bn, (double *)nullptr, rp.data(), (int *)nullptr);
    std::printf("malformed CSR accepted\n");
    failures++;
  } catch (const error &e) {
    if (e.status != WK_ERR_INVALID) failures++;
  }
  std::printf("driver %s: %d failure(s)\n", failures ? "FAILED" : "passed", failures);
  return failures ? 1 : 0;
}

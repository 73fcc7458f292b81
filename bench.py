#!/usr/bin/env python
"""SpMV benchmark: plain fp64 WPK2 `run` on the 3-D trilinear hex mesh of
128^3 elements with 3 dofs per node (6,440,067 rows, 513,599,625 nnz).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one SpMV (engine::run) over the whole matrix.  Prints one JSON
line (rank 0).  `value` is the algorithmic HBM throughput in GB/s
(12 bytes per nnz + 20 bytes per row for fp64 run) with inputs resident in
HBM; `e2e` is the same metric through the library's host-vector call
(H2D of x, SpMV, D2H of y every step, the copies of neighbouring steps
overlapped with each SpMV).  The matrix (6.3 GB) is larger than
L2, so no flush is needed between steps.

--impl reference times the reference path's CPU implementation (the oracle's
restatement of the reference's WPK2 run, OpenMP across warps) on the host
cores for the same workload; under torchrun only rank 0 runs it.

Multi-GPU: one matrix's SpMV is not sharded (one GPU per matrix);
--gpus N runs N independent replicas and reports the sum of their work over
the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SpMV HBM GB/s (% of peak) and nnz/s, fp64 plain vs fp32/bf16 at stated error"
WORKLOAD = dict(name="hex128_3dof_fp64_wpk2_run", dim=3, e=128, dof=3, value_mode=1, seed=1)


def workload(args):
    """The headline workload, or a smaller hex mesh of the same family (--mesh E)."""
    W = dict(WORKLOAD)
    if args.mesh != 128:
        W.update(e=args.mesh, name=f"hex{args.mesh}_3dof_fp64_wpk2_run")
    return W


def alg_bytes(nrows, nnz, mapped=True):
    """fp64 run: 8 B value + 4 B column per nnz; per row 8 B x + 8 B y (+4 B row_map)."""
    return 12 * nnz + (20 if mapped else 16) * nrows


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(kind, threshold):
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    return d.get(f"{kind}_t{threshold}")


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        rows = [ln.split(",") for ln in open(self.f.name).read().splitlines() if ln.strip()]
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, ms_local, world):
    """Whole-job rate of `world` independent replicas: all ranks' units over
    the slowest rank's time (max over ranks)."""
    ms = max_over_ranks(ms_local, world)
    return world * units_per_rank / (ms * 1e-3), ms


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_csr_baseline(rowptr, cols, vals, x, budget_s=10.0, max_reps=50):
    """Oracle CSR multiply (OpenMP, all host threads) on the host copy of the matrix."""
    from oracle import wk_oracle as O
    nthreads = O.max_threads()
    y = O.csr_spmv(rowptr, cols, vals, x, nthreads)  # warm-up (first touch of y)
    times = []
    t_end = time.perf_counter() + budget_s
    while len(times) < max_reps and (not times or time.perf_counter() < t_end):
        t0 = time.perf_counter()
        O.lib().wko_csr_spmv_f64(rowptr, cols, vals, x, y, len(rowptr) - 1, nthreads)
        times.append(time.perf_counter() - t0)
    return statistics.median(times), nthreads, len(times), y


def run_ours(args):
    import numpy as np
    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300 import fe

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    W = workload(args)
    rowptr, cols, vals = fe.fe_matrix(W["dim"], W["e"], W["e"], W["e"], W["dof"], W["value_mode"], W["seed"])
    n, nnz = rowptr.numel() - 1, cols.numel()
    x = fe.uniform_vec(W["seed"], 0, n)
    if args.kind == 1:
        k = wk.structure().scan(nnz, n, vals, rowptr, cols)
    else:
        k = wk.structure2().scan(nnz, n, vals, rowptr, cols, args.threshold)
    eng = wk.engine(k, vals, cols)
    y = torch.zeros(n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    bs = args.blocksize
    nb = (k.nwarps + bs // 32 - 1) // (bs // 32)

    def step():
        eng.run(nb, bs, x, y, cache=True, order=args.order, stream=stream, timed=False)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with Clocks(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(args.steps):
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        t1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    total_ms = max_over_ranks(t0.elapsed_time(t1), world)
    kern_times = [a.elapsed_time(b) for a, b in ev]
    kern_ms = statistics.mean(kern_times)
    clocks = clk.summary()

    B = alg_bytes(n, nnz)
    ms_per_step = total_ms / args.steps
    value = world * B / (ms_per_step * 1e-3) / 1e9
    peak, peak_kind = load_peaks()
    achieved = B / (kern_ms * 1e-3) / 1e9

    # correctness guard against the CSR product computed on the host
    y_host = y.cpu().numpy()
    rp_h, cols_h, vals_h, x_h = (t.cpu().numpy() for t in (rowptr, cols, vals, x))

    # e2e: through the library's host-vector calls.  Each step uploads its x
    # from pinned host memory and downloads its y; wk_run_host_stream overlaps
    # the copies of neighbouring steps with each SpMV (a ring of 4 pinned x / y
    # buffers stands for the stream of host vectors).  The synchronous
    # one-vector call is reported beside it.
    ring = 4
    xhs = [torch.from_numpy(x_h).pin_memory() for _ in range(ring)]
    yhs = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(ring)]
    seq_x = [xhs[i % ring] for i in range(args.steps)]
    seq_y = [yhs[i % ring] for i in range(args.steps)]
    eng.run_host_stream(xhs, yhs, mapped=True, order=args.order)
    barrier(world)
    te = time.perf_counter()
    eng.run_host_stream(seq_x, seq_y, mapped=True, order=args.order)
    e2e_s = max_over_ranks((time.perf_counter() - te) / args.steps, world)
    e2e_value = world * B / e2e_s / 1e9
    e2e_ok = all(bool(np.array_equal(yh.numpy(), y_host)) for yh in yhs)
    xh, yh = xhs[0], yhs[0]
    barrier(world)
    te = time.perf_counter()
    for _ in range(args.steps):
        eng.run_host(xh, yh, mapped=True, order=args.order)
    e2e_sync_s = max_over_ranks((time.perf_counter() - te) / args.steps, world)

    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(ms_per_step, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded FE hex mesh generated on the device)",
        "config": {"workload": W["name"], "mesh": f"hex {W['e']}^3, 3 dof/node, random SPD element blocks",
                   "nrows": n, "nnz": nnz, "layout": "WPK2" if args.kind == 2 else "WPK1",
                   "threshold": args.threshold if args.kind == 2 else None, "nwarps": k.nwarps,
                   "allocate_nz": k.allocate_nz, "order": "fast" if args.order == 0 else "exact",
                   "blocksize": bs, "nblocks": nb, "parallelism": f"replicas{world}",
                   "l2": f"inputs larger than L2 ({B / 1e9:.2f} GB streamed per step), no flush"},
        "nnz_per_s": round(world * nnz / (ms_per_step * 1e-3), 1),
        "gflops": round(world * 2 * nnz / (ms_per_step * 1e-3) / 1e9, 2),
        "pct_of_hbm_peak": round(100 * value / world / peak, 2),
        "clocks": clocks,
        "e2e": {"value": round(e2e_value, 2), "unit": "GB/s", "h2d_bytes_per_step": 8 * n,
                "d2h_bytes_per_step": 8 * n, "ms_per_step": round(e2e_s * 1e3, 4),
                "api": "wk_run_host_stream (pinned host x/y per step, copies overlapped with the SpMV, "
                       "double-buffered)", "y_matches_device_run": e2e_ok,
                "sync_one_vector_call": {"api": "wk_run_host", "value": round(world * B / e2e_sync_s / 1e9, 2),
                                         "ms_per_step": round(e2e_sync_s * 1e3, 4)}},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "traffic": load_traffic(args.kind, args.threshold) if args.mesh == 128 else None,
                     "kernel": "k_spmv_fast<double,MAPPED,L1>", "kernel_ms": round(kern_ms, 5),
                     "kernel_ms_median": round(statistics.median(kern_times), 5),
                     "alg_bytes_per_launch": B},
    }
    if rank == 0 and not args.no_parity:
        # every device-built layout array, the padded arrays, the renumbered
        # columns and x, and the exact-order run against the oracle's host
        # restatement on this matrix (after the timed region)
        from oracle import parity
        y_ex = torch.zeros(n, dtype=torch.float64, device="cuda")
        eng.run(nb, bs, x, y_ex, cache=True, order=1, stream=stream, timed=False)
        torch.cuda.synchronize()
        par = parity.compare(k, eng, rp_h, cols_h, vals_h, x_h, args.kind, args.threshold if args.kind == 2 else 0,
                             y_exact=y_ex.cpu().numpy(), y_fast=y_host, cols_dev=cols, x_dev=x)
        out["parity_c2" if args.mesh == 128 else f"parity_hex{args.mesh}"] = {
            "against": "oracle restatement of the reference's host scan / process / reorderings / run (fma)",
            **par}
        del y_ex
    if rank == 0 and not args.no_cpu_baseline:
        med, nth, reps, y_cpu = cpu_csr_baseline(rp_h, cols_h, vals_h, x_h, budget_s=args.cpu_budget)
        out["cpu_baseline"] = {"value": round(B / med / 1e9, 2), "unit": "GB/s", "cores": nth, "kind": "port",
                               "sample": f"full matrix, {reps} CSR multiplies (oracle wko_csr_spmv_f64, "
                                         f"OpenMP static rows), median {med * 1e3:.2f} ms"}
        nrm = float(np.linalg.norm(y_cpu))
        out["rel_err_vs_host_csr"] = float(np.linalg.norm(y_host - y_cpu) / nrm) if nrm else 0.0
    del eng, k, rowptr, cols, vals, x, y, xh, yh, xhs, yhs, seq_x, seq_y
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_suites:
        out["suites"] = run_suites(args)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return out, rank


# ---- the other rows of the benchmark table ---------------------------------------

def _event_ms(fn, reps, warm=3):
    import torch
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def suite_mixed_and_cg(reps):
    """hex 96^3 (3 dof, seed 2): fp64 vs FP32 / BF16 / scaled-FP16 (WK_F16S)
    stored SpMV with FP32 accumulation (error vs the fp64 host CSR product),
    then fp64 CG vs iterative-refinement CG to 1e-10 with b = A x*."""
    import numpy as np
    import torch

    import warpkernel_gb300 as wk
    from oracle import wk_oracle as O
    from warpkernel_gb300 import fe
    rp, cols, vals = fe.fe_matrix(3, 96, 96, 96, 3, 1, 2)
    n, nnz = rp.numel() - 1, cols.numel()
    x = fe.uniform_vec(2, 0, n)
    y_ref = O.csr_spmv(rp.cpu().numpy(), cols.cpu().numpy(), vals.cpu().numpy(), x.cpu().numpy())
    k = wk.structure2().scan(nnz, n, None, rp, None, 81)
    res = {"workload": "hex96_3dof seed 2", "nrows": n, "nnz": nnz, "paths": {}}
    e64 = wk.engine(k, vals, cols)
    y64 = torch.zeros(n, dtype=torch.float64, device="cuda")
    ms64 = _event_ms(lambda: e64.run(0, 128, x, y64, timed=False), reps)
    base = nnz / ms64
    res["paths"]["f64"] = {"ms": round(ms64, 4), "gnnz_s": round(nnz / ms64 / 1e6, 1), "speedup": 1.0,
                           "gbs": round((12 * nnz + 20 * n) / ms64 / 1e6, 1),
                           "rel_err": float(np.linalg.norm(y64.cpu().numpy() - y_ref) / np.linalg.norm(y_ref))}
    engines = {}
    # (name, value/x tensor type, engine dtype, stored value bytes, x bytes)
    for name, tdt, dt, vb, xb in (("f32", torch.float32, "f32", 4, 4), ("bf16", torch.bfloat16, "bf16", 2, 2),
                                  ("f16s", torch.float32, "f16s", 2, 4)):
        e = wk.engine(k, fe.convert(vals, tdt), cols, dtype=dt)
        xd = fe.convert(x, tdt)
        yd = torch.zeros(n, dtype=torch.float32, device="cuda")
        for comp, win in ((False, False), (True, False), (True, True)):
            if comp:
                e.compress_cols()
                nwin = e.set_windows(win)
            ms = _event_ms(lambda: e.run(0, 128, xd, yd, timed=False), reps)
            err = float(np.linalg.norm(yd.double().cpu().numpy() - y_ref) / np.linalg.norm(y_ref))
            ib = 2 if comp else 4
            res["paths"][name + ("+cols16" if comp else "") + ("+xwin" if win else "")] = {
                "ms": round(ms, 4), "gnnz_s": round(nnz / ms / 1e6, 1), "speedup": round((nnz / ms) / base, 3),
                "gbs": round(((vb + ib) * nnz + (xb + 4 + 4) * n) / ms / 1e6, 1), "rel_err": err,
                **({"window_warps": nwin} if win else {})}
        engines[name] = e
    # CG: b = A x*, x* uniform(-1, 1)
    xs = fe.uniform_vec(2, 1, n)
    b = torch.zeros(n, dtype=torch.float64, device="cuda")
    e64.run(0, 128, xs, b, order=1, timed=False)
    torch.cuda.synchronize()
    xc = torch.zeros_like(b)
    cg = wk.wpk.cg(e64, b, xc, tol=1e-10, max_iter=20000, check_every=16)
    xi = torch.zeros_like(b)
    ir = wk.wpk.ir_cg(e64, engines["f32"], b, xi, tol=1e-10, inner_tol=1e-5, max_inner=20000, check_every=16)
    xi32 = torch.zeros_like(b)
    ir32 = wk.wpk.ir_cg(e64, engines["f32"], b, xi32, tol=1e-10, inner_tol=1e-5, max_inner=20000, check_every=16,
                        inner_dots="fp32")
    xb = torch.zeros_like(b)
    irb = wk.wpk.ir_cg(e64, engines["bf16"], b, xb, tol=1e-10, inner_tol=1e-2, max_inner=20000, check_every=16)
    xh = torch.zeros_like(b)
    irh = wk.wpk.ir_cg(e64, engines["f16s"], b, xh, tol=1e-10, inner_tol=1e-3, max_inner=20000, check_every=16)
    res["cg"] = {"inner_dot_products": "fp64 unless named fp32_dots",
                 "fp64_cg": cg, "ir_cg_f32_inner_fp64_dots": ir, "ir_cg_f32_inner_fp32_dots": ir32,
                 "ir_cg_bf16_inner": irb, "ir_cg_f16s_inner": irh,
                 "ir_f32_speedup": round(cg["seconds"] / ir["seconds"], 3),
                 "ir_f32_fp32_dots_speedup": round(cg["seconds"] / ir32["seconds"], 3),
                 "ir_bf16_speedup": round(cg["seconds"] / irb["seconds"], 3),
                 "ir_f16s_speedup": round(cg["seconds"] / irh["seconds"], 3)}
    return res


def suite_cg(iters, mesh=96):
    """Profiling case: one fp64 CG of `iters` iterations (16-iteration graph
    batches) on hex mesh^3 (3 dof, seed 2, WPK2 th=81), then one plain SpMV."""
    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300 import fe
    rp, cols, vals = fe.fe_matrix(3, mesh, mesh, mesh, 3, 1, 2)
    n, nnz = rp.numel() - 1, cols.numel()
    k = wk.structure2().scan(nnz, n, None, rp, None, 81)
    e64 = wk.engine(k, vals, cols)
    xs = fe.uniform_vec(2, 1, n)
    b = torch.zeros(n, dtype=torch.float64, device="cuda")
    e64.run(0, 128, xs, b, order=1, timed=False)
    x = torch.zeros_like(b)
    res = wk.wpk.cg(e64, b, x, tol=1e-30, max_iter=iters, check_every=16)
    y = torch.zeros_like(b)
    spmv = e64.run(0, 128, xs, y)
    return {"workload": f"hex{mesh}_3dof fp64 CG", "nrows": n, "nnz": nnz, "cg": res,
            "ms_per_iteration": round(res["seconds"] * 1e3 / max(res["iters"], 1), 4),
            "spmv_ms": round(spmv * 1e3, 4)}


def suite_adjoint(reps):
    """hex 64^3 (3 dof, seed 4), fp32: forward SpMV vs forward + adjoint
    (dx = A^T dy and dvals) through the autograd binding's kernels."""
    import torch

    from warpkernel_gb300 import fe
    from warpkernel_gb300.autograd import WPKMatrix
    rp, cols, vals = fe.fe_matrix(3, 64, 64, 64, 3, 1, 4)
    n, nnz = rp.numel() - 1, cols.numel()
    x = fe.uniform_vec(4, 0, n).float()
    dy = fe.uniform_vec(4, 2, n).float()
    out = {"workload": "hex64_3dof fp32 seed 4", "nrows": n, "nnz": nnz}
    for order in ("slots", "csr"):
        v = vals.float()
        m0 = WPKMatrix(rp, cols, v, kind=2, threshold=81)
        mat = m0 if order == "csr" else WPKMatrix(rp, cols, m0.to_slots(v), kind=2, threshold=81,
                                                  value_order="slots")
        y = torch.zeros(n, dtype=torch.float32, device="cuda")

        def fwd():
            mat.eng.run(0, 128, x, y, timed=False)

        def adj():
            mat.adjoint(x, dy)

        tf = _event_ms(fwd, reps)
        ta = _event_ms(adj, reps)
        tb = _event_ms(lambda: (fwd(), adj()), reps)
        out[order] = {"fwd_ms": round(tf, 4), "adj_ms": round(ta, 4), "fwd_plus_adj_ms": round(tb, 4),
                      "ratio": round(tb / tf, 3), "fused_symmetric_path": mat.symmetric}
        if order == "slots":
            # dx = A^T dy alone (no dvals): the adjoint a linear solve's gradient needs
            def adj_dx():
                mat.adjoint(x, dy, want_dx=True, want_dvals=False)

            td = _event_ms(adj_dx, reps)
            tbd = _event_ms(lambda: (fwd(), adj_dx()), reps)
            out["dx_only"] = {"fwd_ms": round(tf, 4), "adj_ms": round(td, 4), "fwd_plus_adj_ms": round(tbd, 4),
                              "ratio": round(tbd / tf, 3)}
            # the same pair with 16-bit columns on both sides
            mat.eng.compress_cols()
            tf = _event_ms(fwd, reps)
            ta = _event_ms(adj, reps)
            tb = _event_ms(lambda: (fwd(), adj()), reps)
            out["slots+cols16"] = {"fwd_ms": round(tf, 4), "adj_ms": round(ta, 4), "fwd_plus_adj_ms": round(tb, 4),
                                   "ratio": round(tb / tf, 3)}
    # a general (unsymmetric) pattern: the same matrix with 1 % of its
    # off-diagonal entries dropped (seed 5), so the adjoint takes the
    # transposed engine's SpMV for dx and a second pass for dvals
    gen = torch.Generator(device="cuda").manual_seed(5)
    rpc = rp.to("cuda", torch.int64)
    rows = torch.repeat_interleave(torch.arange(n, device="cuda"), rpc[1:] - rpc[:-1])
    cc = cols.to("cuda", torch.int64)
    keep = (rows == cc) | (torch.rand(nnz, device="cuda", generator=gen) > 0.01)
    rows_k = rows[keep]
    rp_k = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    rp_k[1:] = torch.cumsum(torch.bincount(rows_k, minlength=n), 0)
    v_k = vals.to("cuda")[keep].float()
    g_csr = WPKMatrix(rp_k.to(torch.int32), cc[keep].to(torch.int32), v_k, kind=2, threshold=81)
    g_slot = WPKMatrix(rp_k.to(torch.int32), cc[keep].to(torch.int32), g_csr.to_slots(v_k), kind=2, threshold=81,
                       value_order="slots")
    y = torch.zeros(n, dtype=torch.float32, device="cuda")
    tf = _event_ms(lambda: g_csr.eng.run(0, 128, x, y, timed=False), reps)
    out["general_pattern"] = {"nnz": int(keep.sum().item()), "symmetric": g_csr.symmetric, "fwd_ms": round(tf, 4)}
    for order, m in (("csr", g_csr), ("slots", g_slot)):
        ta = _event_ms(lambda: m.adjoint(x, dy), reps)
        out["general_pattern"][f"{order}_adj_ms"] = round(ta, 4)
    return out


def suite_f16s(reps, mesh=96, dtype="f16s", cols16=False, windows=True):
    """hex mesh^3 (3 dof, seed 2, WPK2 threshold 81): one stored-value engine
    alone (`dtype` f16s: scaled FP16 values with FP32 x and y; f32; bf16 with
    bf16 x and FP32 y), optionally with 16-bit columns.  GB/s counts value +
    column bytes per nonzero and x + y + row map bytes per row."""
    import numpy as np
    import torch

    import warpkernel_gb300 as wk
    from oracle import wk_oracle as O
    from warpkernel_gb300 import fe
    rp, cols, vals = fe.fe_matrix(3, mesh, mesh, mesh, 3, 1, 2)
    n, nnz = rp.numel() - 1, cols.numel()
    x = fe.uniform_vec(2, 0, n)
    k = wk.structure2().scan(nnz, n, None, rp, None, 81)
    tdt, vb, xb = {"f16s": (torch.float32, 2, 4), "f32": (torch.float32, 4, 4), "bf16": (torch.bfloat16, 2, 2)}[dtype]
    e = wk.engine(k, fe.convert(vals, tdt), cols, dtype=dtype)
    nwin = 0
    if cols16:
        e.compress_cols()
        nwin = e.set_windows(windows)
    xd = fe.convert(x, tdt)
    yd = torch.zeros(n, dtype=torch.float32, device="cuda")
    ms = _event_ms(lambda: e.run(0, 128, xd, yd, timed=False), reps)
    y_ref = O.csr_spmv(rp.cpu().numpy(), cols.cpu().numpy(), vals.cpu().numpy(), x.cpu().numpy())
    err = float(np.linalg.norm(yd.double().cpu().numpy() - y_ref) / np.linalg.norm(y_ref))
    ib = 2 if cols16 else 4
    return {"workload": f"hex{mesh}_3dof seed 2 {dtype}" + ("+cols16" if cols16 else "") + ("+xwin" if nwin else ""),
            "window_warps": nwin, "nrows": n, "nnz": nnz,
            "ms": round(ms, 4), "gbs": round(((vb + ib) * nnz + (xb + 8) * n) / ms / 1e6, 1), "rel_err": err}


def suite_permuted(reps, mesh=128):
    """The headline matrix (hex mesh^3, 3 dof, seed 1) under a seeded random
    symmetric permutation of rows and columns (A' = P A P^T, columns sorted
    within rows): the FE locality of the x gathers is gone, x (8 B x n) stays
    L2-resident.  fp64 WPK2 threshold 81 `run`, algorithmic GB/s (12 B/nnz +
    20 B/row) beside the unpermuted matrix; y' checked against the
    unpermuted product under the permutation."""
    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300 import fe
    rp, cols, vals = fe.fe_matrix(3, mesh, mesh, mesh, 3, 1, 1)
    n, nnz = rp.numel() - 1, cols.numel()
    x = fe.uniform_vec(1, 0, n)
    out = {"workload": f"hex{mesh}_3dof fp64 seed 1, random symmetric permutation (torch.randperm, seed 1)",
           "nrows": n, "nnz": nnz}

    def measure(rp_, cols_, vals_, x_):
        k = wk.structure2().scan(nnz, n, None, rp_, None, 81)
        e = wk.engine(k, vals_, cols_)
        y = torch.zeros(n, dtype=torch.float64, device="cuda")
        ms = _event_ms(lambda: e.run(0, 128, x_, y, timed=False), reps)
        del e, k
        return ms, y

    ms0, y0 = measure(rp, cols, vals, x)
    g = torch.Generator(device="cuda")
    g.manual_seed(1)
    perm = torch.randperm(n, device="cuda", generator=g)  # row i of A -> row perm[i] of A'
    lens = (rp[1:] - rp[:-1]).long()
    rows = torch.repeat_interleave(torch.arange(n, device="cuda"), lens)
    key = perm[rows] * n + perm[cols.long()]
    del rows
    key, order = torch.sort(key)
    cols_p = (key % n).to(torch.int32)
    del key
    vals_p = vals[order]
    del order
    lens_p = torch.empty_like(lens)
    lens_p[perm] = lens
    rp_p = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    rp_p[1:] = torch.cumsum(lens_p, 0).to(torch.int32)
    x_p = torch.empty_like(x)
    x_p[perm] = x
    del lens, lens_p
    torch.cuda.empty_cache()
    ms1, y1 = measure(rp_p, cols_p, vals_p, x_p)
    err = float((y1[perm] - y0).norm() / y0.norm())
    B = 12 * nnz + 20 * n
    out["natural_order"] = {"ms": round(ms0, 4), "gbs": round(B / ms0 / 1e6, 1)}
    out["permuted"] = {"ms": round(ms1, 4), "gbs": round(B / ms1 / 1e6, 1), "rel_err_vs_natural": err}
    del rp_p, cols_p, vals_p, x_p, y0, y1, perm
    torch.cuda.empty_cache()
    return out


def suite_setup(mesh=128, host=False):
    """Layout and engine construction for the headline matrix (hex mesh^3,
    3 dof, seed 1, WPK2 threshold 81): the device scan (sort, split, offsets,
    reorder_rows) and the device process (padded values and columns), best of
    3 after one warm-up, host clock around synchronised calls.  With `host`,
    the oracle's single-threaded restatement of the reference's host scan and
    process on the same matrix (what the reference does before every run)."""
    import ctypes as C

    import numpy as np
    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300 import fe
    rp, cols, vals = fe.fe_matrix(3, mesh, mesh, mesh, 3, 1, 1)
    n, nnz = rp.numel() - 1, cols.numel()

    def once():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        k = wk.structure2().scan(nnz, n, None, rp, None, 81)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e = wk.engine(k, vals, cols)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        del e, k
        return t1 - t0, t2 - t1

    once()
    t = [once() for _ in range(3)]
    out = {"workload": f"hex{mesh}_3dof fp64 seed 1, WPK2 threshold 81", "nrows": n, "nnz": nnz,
           "device": {"scan_ms": round(min(a for a, _ in t) * 1e3, 2),
                      "process_ms": round(min(b for _, b in t) * 1e3, 2)}}
    if host:
        from oracle import wk_oracle as O
        rp_h = np.ascontiguousarray(rp.cpu().numpy())
        cols_h = np.ascontiguousarray(cols.cpu().numpy())
        vals_h = np.ascontiguousarray(vals.cpu().numpy())
        L = O.lib()
        c = O._Layout()
        t0 = time.perf_counter()
        rc = L.wko_scan2(rp_h, n, nnz, 81, C.byref(c))
        t1 = time.perf_counter()
        if rc == 0:
            pv = np.zeros(c.allocate_nz, np.float64)
            pc = np.zeros(c.allocate_nz, np.int32)
            t2 = time.perf_counter()
            L.wko_process_f64(C.byref(c), vals_h, cols_h, pv, pc)
            t3 = time.perf_counter()
            out["host_oracle_1_thread"] = {"scan_s": round(t1 - t0, 3), "process_s": round(t3 - t2, 3)}
        L.wko_free(C.byref(c))
    return out


def _graph_us(fn, launches=100, replays=20):
    """Microseconds per call of `fn` (stream-ordered launches on the current
    stream), from CUDA-graph replays of `launches` calls, CUDA events around
    `replays` replays."""
    import torch
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(3):
            fn()
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(launches):
            fn()
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(replays):
        g.replay()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) * 1e3 / (replays * launches)


def suite_small():
    """2-D Q1 128^2, 1 dof (16,641 rows, 148,225 nnz, rows of 9/6/4, seed 0),
    fp64: run (original columns, y scattered through row_map) and run_x
    (coalesced renumbered columns, reordered x, y in sorted order) for WPK1
    and WPK2 thresholds 2-8, fast and exact order.  The 2 MB matrix stays in
    L2, so this reports latency and GFLOP/s (2 flops per nonzero) from
    CUDA-graph replays, not an HBM fraction."""
    import numpy as np
    import torch

    import warpkernel_gb300 as wk
    from oracle import wk_oracle as O
    from warpkernel_gb300 import fe
    rp, cols, vals = fe.fe_matrix(2, 128, 128, 0, 1, 0, 0)
    n, nnz = rp.numel() - 1, cols.numel()
    x = fe.uniform_vec(0, 0, n)
    y_ref = O.csr_spmv(rp.cpu().numpy(), cols.cpu().numpy(), vals.cpu().numpy(), x.cpu().numpy())
    out = {"workload": "q1_128x128_1dof fp64 seed 0 (L2-resident)", "nrows": n, "nnz": nnz,
           "timing": "CUDA graph of 100 launches, 20 replays", "layouts": {}}
    for name, th in (("wpk1", None), ("wpk2_th8", 8), ("wpk2_th5", 5), ("wpk2_th3", 3), ("wpk2_th2", 2)):
        k = wk.structure().scan(nnz, n, None, rp) if th is None else wk.structure2().scan(nnz, n, None, rp, None, th)
        e = wk.engine(k, vals, cols)
        ex = wk.engine(k, vals, cols)
        ex.device_colinds = k.reorder_columns_coalesced(cols)
        xr = k.reorder_x(x)
        y = torch.zeros(n, dtype=torch.float64, device="cuda")
        yx = torch.zeros(n, dtype=torch.float64, device="cuda")
        row = {"nwarps": k.nwarps, "allocate_nz": k.allocate_nz}
        for order, oname in ((0, "fast"), (1, "exact")):
            us = _graph_us(lambda: e.run(0, 128, x, y, order=order, timed=False))
            usx = _graph_us(lambda: ex.run_x(0, 128, xr, yx, order=order, timed=False))
            torch.cuda.synchronize()
            err = float(np.linalg.norm(y.cpu().numpy() - y_ref) / np.linalg.norm(y_ref))
            rm = torch.from_numpy(k.row_map.astype(np.int64)).cuda()
            same = bool(torch.equal(yx, y[rm]))
            row[oname] = {"run_us": round(us, 2), "run_gflops": round(2 * nnz / us / 1e3, 1),
                          "run_x_us": round(usx, 2), "run_x_gflops": round(2 * nnz / usx / 1e3, 1),
                          "rel_err": err, "run_x_equals_run": same}
        out["layouts"][name] = row
    return out


def suite_batched(count=512, tune=True):
    """512 FE patches (2-D Q1 / 3-D hex, 1k-200k rows, 1 or 3 dof, 1-16 RHS,
    fp32, seed 3) in one persistent CUDA-graph launch; autotuned threshold
    and RHS tile (tuned on the whole set: on the first 128 matrices alone the
    choice flipped between runs to a threshold that is 33 % slower on all 512)."""
    import torch

    from warpkernel_gb300 import batched
    specs = batched.fe_matrix_set(512, seed=3)[:count]
    tune = batched.autotune(specs, reps=5) if tune else {"threshold_frac": 1.0, "rhs_tile": 16}
    b = batched.Batch.from_fe(specs, "f32", tune["threshold_frac"], tune["rhs_tile"])
    X, Y = batched.make_vectors(specs)
    b.set_vectors(X, Y)
    b.capture()
    secs = sorted(b.run() for _ in range(10))
    med = secs[len(secs) // 2]
    B = batched.algorithmic_bytes(specs)
    nnz_rhs = sum(s["nnz"] * s["nrhs"] for s in specs)
    del b, X, Y
    torch.cuda.empty_cache()
    return {"matrices": len(specs), "rows": sum(s["nrows"] for s in specs), "nnz": sum(s["nnz"] for s in specs),
            "nnz_rhs": nnz_rhs, "ms": round(med * 1e3, 4), "gnnz_rhs_s": round(nnz_rhs / med / 1e9, 2),
            "gbs": round(B / med / 1e9, 1), "threshold_frac": tune["threshold_frac"], "rhs_tile": tune["rhs_tile"],
            "launch": "one persistent kernel, CUDA graph replay"}


def powerlaw_csr(n, seed=5, zipf=1.6, maxlen=2000, band=4096):
    """Seeded skewed matrix: row lengths from a Zipf law (1..maxlen), columns
    uniform within a band around the diagonal (unsorted, duplicates allowed)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    lens = np.minimum(rng.zipf(zipf, n), maxlen).astype(np.int64)
    rp = np.zeros(n + 1, np.int64)
    rp[1:] = np.cumsum(lens)
    rows = np.repeat(np.arange(n, dtype=np.int64), lens)
    cols = np.clip(rows + rng.integers(-band, band + 1, int(rp[-1])), 0, n - 1)
    vals = rng.uniform(-1, 1, int(rp[-1]))
    return rp.astype(np.int32), cols.astype(np.int32), vals


def suite_ablation(reps):
    """The optimization.cu ablation on GB300: WPK1 (sorted, interleaved) vs
    scan_nosort, scan_nocoalesced and both, fp64 run, on the hex 64^3 FE matrix
    (near-uniform rows) and a seeded power-law matrix (skewed rows); WPK2 at
    the best of a few thresholds beside them.  GB/s counts the matrix's own
    12 B/nnz + 20 B/row, so padding shows up as lost throughput."""
    import torch

    import warpkernel_gb300 as wk
    from warpkernel_gb300 import fe
    out = {}
    mats = {"hex64_3dof": None, "powerlaw_1M": None}
    for name in mats:
        if name == "hex64_3dof":
            rp, cols, vals = (t.cpu().numpy() for t in fe.fe_matrix(3, 64, 64, 64, 3, 1, 4))
        else:
            rp, cols, vals = powerlaw_csr(1 << 20)
        n, nnz = len(rp) - 1, len(cols)
        x = fe.uniform_vec(4, 0, n)
        y = torch.zeros(n, dtype=torch.float64, device="cuda")
        B = alg_bytes(n, nnz)
        rows = {}

        def timed(eng, order):
            return _event_ms(lambda: eng.run(0, 128, x, y, order=order, timed=False), reps)

        for label, flags in (("wpk1", 0), ("nosort", 1), ("nocoalesced", 2), ("nocoalesced_nosort", 3)):
            k = wk.structure().scan_ablation(nnz, n, rp, flags) if flags else wk.structure().scan(nnz, n, None, rp)
            eng = wk.engine(k, vals, cols)
            r = {"padding": round(k.allocate_nz / nnz, 4)}
            for oname, order in (("exact", 1), ("fast", 0)):
                if flags & 2 and order == 0:
                    continue  # one order only
                ms = timed(eng, order)
                r[oname] = {"ms": round(ms, 4), "gbs": round(B / ms / 1e6, 1)}
            rows[label] = r
            del eng, k
        best = None
        for th in (8, 32, 81, 256):
            k = wk.structure2().scan(nnz, n, None, rp, None, th)
            eng = wk.engine(k, vals, cols)
            ms = timed(eng, 0)
            if best is None or ms < best["ms"]:
                best = {"threshold": th, "ms": round(ms, 4), "gbs": round(B / ms / 1e6, 1),
                        "padding": round(k.allocate_nz / nnz, 4)}
            del eng, k
        rows["wpk2_best_fast"] = best
        out[name] = {"nrows": n, "nnz": nnz, **rows}
        torch.cuda.empty_cache()
    return out


def run_suites(args):
    import torch
    out = {}
    for name, fn in (("mixed_precision_and_cg", lambda: suite_mixed_and_cg(50)),
                     ("adjoint", lambda: suite_adjoint(50)), ("batched", suite_batched),
                     ("ablation", lambda: suite_ablation(20)), ("small_q1_128", suite_small),
                     ("permuted_hex128", lambda: suite_permuted(20)),
                     ("setup_hex128", suite_setup)):
        t0 = time.time()
        try:
            out[name] = fn()
        except Exception as e:  # a failing suite must not hide the headline
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["wall_s"] = round(time.time() - t0, 2)
        torch.cuda.empty_cache()
    return out


def run_reference(args):
    """The reference path's arithmetic on the host cores: oracle scan + WPK
    run in the reference's order, OpenMP across warps."""
    import numpy as np

    from oracle import wk_oracle as O

    world, rank, _ = dist_setup()
    if rank != 0:
        return None, rank
    W = workload(args)
    rowptr, cols, vals = O.fe_matrix(W["dim"], W["e"], W["e"], W["e"], W["dof"], W["value_mode"], W["seed"])
    n, nnz = len(rowptr) - 1, len(cols)
    x = O.uniform_vec(W["seed"], 0, n)
    o = O.OracleLayout(rowptr, kind=args.kind, threshold=args.threshold)
    pv, pc = o.process(vals, cols)
    del vals, cols
    y = np.zeros(n)
    nth = O.max_threads()
    for _ in range(max(args.warmup, 3)):
        o.run_omp(pv, pc, x, y, nth)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.run_omp(pv, pc, x, y, nth)
        times.append(time.perf_counter() - t0)
    B = alg_bytes(n, nnz)
    ms = statistics.mean(times) * 1e3
    value = B / (ms * 1e-3) / 1e9
    out = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded FE hex mesh generated on the host)",
        "config": {"workload": W["name"], "nrows": n, "nnz": nnz,
                   "layout": "WPK2" if args.kind == 2 else "WPK1",
                   "threshold": args.threshold if args.kind == 2 else None},
        "nnz_per_s": round(nnz / (ms * 1e-3), 1),
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": nth, "kind": "port",
                         "sample": f"full matrix per step, {args.steps} WPK run passes (oracle restatement "
                                   "of the reference's run, OpenMP across warps)"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own GPU path (CUDA 4.0 texture references, sm_30) does not build with CUDA 13",
    }
    return out, rank


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--kind", type=int, default=2, choices=[1, 2])
    ap.add_argument("--threshold", type=int, default=81)
    ap.add_argument("--order", type=int, default=0, choices=[0, 1])
    ap.add_argument("--blocksize", type=int, default=128)
    ap.add_argument("--mesh", type=int, default=128, help="hex elements per axis (128 = the headline)")
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the full-size comparison of the layout and run with the oracle")
    ap.add_argument("--no-suites", action="store_true",
                    help="skip the mixed-precision / CG / adjoint / batched measurements")
    ap.add_argument("--value-dtype", choices=["f16s", "f32", "bf16"], default="f16s",
                    help="--only f16s: the stored value type")
    ap.add_argument("--cols16", action="store_true", help="--only f16s: 16-bit column storage")
    ap.add_argument("--no-windows", action="store_true", help="--only f16s: 16-bit columns without x windows")
    ap.add_argument("--only", choices=["mixed", "adjoint", "batched", "ablation", "cg", "f16s", "small", "permuted", "setup"],
                    help="run one suite alone (profiling cases; --steps = timed repetitions, "
                         "batched: the first 128 matrices with a fixed threshold / tile)")
    args = ap.parse_args()
    if args.only:
        import torch
        torch.cuda.set_device(0)
        reps = max(args.steps, 1)
        if args.only == "mixed":
            res = suite_mixed_and_cg(reps)
        elif args.only == "adjoint":
            res = suite_adjoint(reps)
        elif args.only == "ablation":
            res = suite_ablation(reps)
        elif args.only == "cg":
            res = suite_cg(reps, args.mesh)
        elif args.only == "f16s":
            res = suite_f16s(reps, args.mesh, args.value_dtype, args.cols16, not args.no_windows)
        elif args.only == "small":
            res = suite_small()
        elif args.only == "permuted":
            res = suite_permuted(reps, args.mesh)
        elif args.only == "setup":
            res = suite_setup(args.mesh, host=True)
        else:
            res = suite_batched(count=128, tune=False)
        print(json.dumps({"suite": args.only, **res}), flush=True)
        return
    if args.impl == "reference":
        out, rank = run_reference(args)
    else:
        out, rank = run_ours(args)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()

"""Benchmarks of the frequency-domain FEM hot path on one GPU; prints one JSON line.

Assembly (the line's metric/value; the reference's assembly micro-benchmark): unit
cube, 80³ hexes × 6 Kuhn tets (3,072,000 tets), interior vertices jittered by
U[-0.15h, 0.15h] (numpy default_rng(0)); per tet εr ~ U[1,10], tanδ ~ U[0.001,0.02]
(default_rng(1)), μr = 1.  One step = assembling the complex128 curl-curl (E) and
mass (B) CSR matrices, i.e. tet_mass_stiffness_matrices
(fem/physics/edm/optimized_assembly.py:43-64).  The CSR pattern is built once per
mesh before timing (reported separately as ``plan_s``).  ``value``: tets/s with
inputs resident in HBM (each step writes 27.5 GB of values, far more than the 129 MB
L2, so no L2 flush is needed).  ``e2e``: the same through the C-ABI host entry point
(emg_assemble_tet_host), with the material H2D and the E/B D2H inside the timed
region; with the bench's page-locked outputs the fill stores straight into them.
``--impl reference`` times the reference's CPU algorithm (the oracle's C++
restatement of the Numba element loop on all host cores + SciPy
coo_matrix(...).tocsr()) on a bounded sample of the same workload.  Under torchrun
(N > 1) every rank assembles its own copy (replicas, weak scaling); the time is the
slowest rank's.

Also reported: ``topology`` (the mesh's edge/face topology and DOF map on the GPU
against the NumPy host build), ``farfield`` (Stratton-Chu transform against its FP32
compute roofline and the NumPy restatement), ``sweep`` (the five-cavity iris filter,
401 points over 8-12 GHz x 2 ports: the batched mixed-precision warm-started GPU sweep
against the plain FP64 GPU solver, with the MLP and cold variants; see run_sweep) and
``eigen`` (cavity eigenmodes against ARPACK; see run_eigen).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--n 80] [--impl reference]
                  [--no-sweep] [--sweep-h 2e-3] [--eigen 2] [--sweep-only] [--eigen-only]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "assembly tets/s (E+B complex128 CSR, 2nd-order Nedelec)"
C0 = 299792458.0


def make_workload(n: int):
    from emerge_gb300.mesh import Nedelec2Basis, unit_cube
    m = unit_cube(n, jitter=0.15, seed=0)
    field = Nedelec2Basis(m)
    rng = np.random.default_rng(1)
    nT = m.n_tets
    er_s = rng.uniform(1.0, 10.0, nT) * (1 - 1j * rng.uniform(0.001, 0.02, nT))
    return m, field, er_s.astype(np.complex128)


def dense_materials(er_s: np.ndarray):
    nT = er_s.shape[0]
    er = np.zeros((3, 3, nT), dtype=np.complex128)
    ur = np.zeros((3, 3, nT), dtype=np.complex128)
    for k in range(3):
        er[k, k] = er_s
        ur[k, k] = 1.0
    return er, ur


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        smax = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def issue_floor_ms(warp_inst: float, clocks: dict) -> float:
    """Time to issue ``warp_inst`` warp instructions on 152 SMs x 4 schedulers at the SM
    clock sampled during the timed region (its maximum when no sample was taken)."""
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    return warp_inst / (152 * 4 * mhz * 1e6) * 1e3


def traffic_per_launch(n: int):
    """DRAM bytes per fill launch from the committed ncu summary (scaled by tets), or None."""
    p = os.path.join(ROOT, "profiles", "assembly_fill_traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    return float(d["dram_bytes_per_tet"]) * 6 * n ** 3


def cpu_reference(field, er_s, max_tets: int):
    """Oracle (C++ restatement of _matrix_builder, OpenMP) + SciPy tocsr on a leading slice of tets."""
    import oracle
    from scipy.sparse import coo_matrix
    nT = min(max_tets, field.mesh.n_tets)
    er, ur = dense_materials(er_s)
    N = field.n_field
    t0 = time.perf_counter()
    dE, dB, rows, cols = oracle.matrix_builder(field, er, ur, 0, nT)
    t1 = time.perf_counter()
    E = coo_matrix((dE, (rows, cols)), shape=(N, N)).tocsr()
    B = coo_matrix((dB, (rows, cols)), shape=(N, N)).tocsr()
    t2 = time.perf_counter()
    del E, B
    return nT, t1 - t0, t2 - t1


def run_reference(args, rank, world):
    if rank != 0:
        return
    n = args.n
    m, field, er_s = make_workload(n)
    cores = os.cpu_count()
    sample = args.cpu_sample
    for _ in range(args.warmup):
        cpu_reference(field, er_s, min(sample, 20000))
    times = []
    nts = None
    for _ in range(args.steps):
        nts, ti, tc = cpu_reference(field, er_s, sample)
        times.append(ti + tc)
    t = sum(times) / len(times)
    v = nts / t
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "tets/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": f"assembly {n}^3 Kuhn unit cube, jitter 0.15h, eps U[1,10] tan U[.001,.02], mu=1",
                   "tets": int(m.n_tets), "n_field": int(field.n_field), "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": v, "unit": "tets/s", "cores": cores, "kind": "port",
                         "sample": f"first {nts} tets of the {n}^3 mesh per step: C++/OpenMP restatement of "
                                   f"_matrix_builder + scipy coo.tocsr (Numba is not available)"},
        "e2e": {"value": v, "unit": "tets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# FP64 flops per tet of the factored isotropic element blocks plus the complex
# material scaling and accumulation (36 ee x 40 + 48 ef/fe x 73 + 16 ff x 129 + 100 x 36)
FP64_TFLOPS = 1.18         # GB300 FP64 FMA throughput measured by a probe kernel (DFMA chain)
FP32_TFLOPS = 74.8         # GB300 FP32 FMA throughput measured by a probe kernel
# warp instructions per tet of one fill (k_elem 1274 + k_fill_st 3570), from the ncu
# capture summarised in profiles/k_elem_k_fill_st_cube40.md; the fill runs on the FP32 and
# integer pipes, so its compute bound is the issue rate of 152 SMs x 4 schedulers
FILL_WARP_INST_PER_TET = 4844


def run_gpu(args, rank, world):
    import torch
    from emerge_gb300 import _build
    from emerge_gb300.assembly import AssemblyPlan, material_scalars
    from emerge_gb300.replicas import max_over_ranks
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    _build.build()
    n = args.n
    m, field, er_s = make_workload(n)
    er, ur = dense_materials(er_s) if n <= 40 else (None, None)
    eps = er_s
    mu_inv = np.ones(m.n_tets, dtype=np.complex128)
    if er is not None:
        eps, mu_inv = material_scalars(er, ur)
    dev = torch.device("cuda", local)
    t0 = time.perf_counter()
    plan = AssemblyPlan(field, dev)
    torch.cuda.synchronize()
    plan_s = time.perf_counter() - t0
    e = torch.as_tensor(eps, device=dev)
    mi = torch.as_tensor(mu_inv, device=dev)
    E = torch.empty(plan.nnz, dtype=torch.complex128, device=dev)
    B = torch.empty(plan.nnz, dtype=torch.complex128, device=dev)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        plan.assemble(e, mi, E, B)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t_begin = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_begin.record(stream)
        for k in range(args.steps):
            starts[k].record(stream)
            plan.assemble(e, mi, E, B)
            ends[k].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize()
        time.sleep(0.3)
    total_ms = t_begin.elapsed_time(t_end)
    launch_ms = [s.elapsed_time(x) for s, x in zip(starts, ends)]
    # replicas: every rank assembles its own copy of the workload (weak scaling); the
    # job's time is the slowest rank's
    ms = max_over_ranks(total_ms / args.steps, device=dev)
    value = world * m.n_tets / (ms / 1e3)

    # end to end through the host entry point: materials H2D + E/B D2H inside the timed region
    pin_E = torch.empty(plan.nnz, dtype=torch.complex128, pin_memory=True)
    pin_B = torch.empty(plan.nnz, dtype=torch.complex128, pin_memory=True)
    pin_eps = torch.as_tensor(eps).pin_memory()
    pin_mu = torch.as_tensor(mu_inv).pin_memory()
    npE, npB = pin_E.numpy(), pin_B.numpy()
    npe, npm = pin_eps.numpy(), pin_mu.numpy()
    for _ in range(max(1, min(args.warmup, 2))):
        plan.assemble_host(npe, npm, npE, npB)
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        plan.assemble_host(npe, npm, npE, npB)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, device=dev)
    e2e_val = world * m.n_tets / e2e_s

    # parity of this very workload against the oracle, on row blocks (untimed)
    parity = assembly_parity(field, er_s, plan, E, B) if rank == 0 and not args.no_cpu else None

    # first call of the drop-in on a new mesh: plan (incidence, CSR pattern, geometry
    # records) + fill + D2H of values and pattern, the work one tet_mass_stiffness_matrices
    # call does before it wraps the host arrays as scipy CSR
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan2 = AssemblyPlan(field, dev)
    plan2.assemble_host(npe, npm, npE, npB)
    plan2.pattern_host()
    first_s = time.perf_counter() - t0
    del plan2

    nnz, nT, nN = plan.nnz, m.n_tets, m.n_nodes
    alg_bytes = 2 * 16 * nnz + 4 * nnz + nT * (20 * 4 + 4 * 4 + 16 + 16) + 24 * nN
    kern_s = statistics.median(launch_ms) / 1e3
    achieved = alg_bytes / kern_s / 1e9
    peak, peak_kind = peaks()
    out = {
        "metric": METRIC, "value": value, "unit": "tets/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "float-float (FP32 pairs, ~48-bit) arithmetic, complex128 storage",
        "data": "synthetic",
        "config": {"workload": f"assembly {n}^3 Kuhn unit cube, jitter 0.15h, eps U[1,10] tan U[.001,.02], mu=1",
                   "tets": int(nT), "n_field": int(plan.n_field), "nnz_per_matrix": int(nnz),
                   "l2": "no flush: each step writes 32*nnz bytes >> 129 MB L2", "parallelism": f"replicas x{world}",
                   "plan_s": round(plan_s, 3)},
        "e2e": {"value": e2e_val, "unit": "tets/s", "h2d_bytes_per_step": int(2 * 16 * nT),
                "d2h_bytes_per_step": int(2 * 16 * nnz), "steps": e2e_steps},
        "first_call": {"value": nT / first_s, "unit": "tets/s", "seconds": round(first_s, 4),
                       "what": "new plan (pattern + records) + fill + D2H of values and pattern, one call"},
        "parity": parity,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     "kernel": "one assembly step: k_scales + k_elem + k_fill_st (+ its Im E pass, empty for real mu)",
                     "algorithmic_bytes_per_launch": int(alg_bytes), "traffic": traffic_per_launch(n),
                     # the float-float arithmetic runs on the FP32/integer pipes: its bound is the
                     # warp-instruction issue rate at the sampled SM clock
                     "compute": {"bound": "issue (FP32 float-float)", "warp_inst_per_tet": FILL_WARP_INST_PER_TET,
                                 "floor_ms": issue_floor_ms(FILL_WARP_INST_PER_TET * nT, clk.summary()),
                                 "frac": issue_floor_ms(FILL_WARP_INST_PER_TET * nT, clk.summary())
                                 / statistics.median(launch_ms)}},
        "gpu_launches": 4 * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0:
        out["topology"] = run_topology(m, n, dev)
        out["farfield"] = run_farfield(dev)
    if rank == 0 and not args.no_sweep:
        del E, B, pin_E, pin_B, npE, npB, plan
        torch.cuda.empty_cache()
        out["sweep"] = run_sweep(args)
    if rank == 0 and args.eigen > 0:
        torch.cuda.empty_cache()
        out["eigen"] = run_eigen(args)
    if rank == 0 and not args.no_cpu:
        nts, ti, tc = cpu_reference(field, er_s, args.cpu_sample)
        out["cpu_baseline"] = {"value": nts / (ti + tc), "unit": "tets/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": f"first {nts} tets of the same mesh: C++/OpenMP restatement of the "
                                         f"reference element loop ({ti:.2f} s) + scipy coo.tocsr ({tc:.2f} s)"}
    if rank == 0:
        print(json.dumps(out))


def assembly_parity(field, er_s, plan, E, B, seed: int = 5):
    """The fill's E and B on row blocks of this mesh against the oracle (pattern bit-exact,
    values relative to each row's largest entry): 5000 random rows plus 2048 contiguous
    rows at the start, the middle and the end of the DOF numbering.  The oracle runs the
    reference's element loop on exactly the tets that touch those rows (untimed)."""
    import oracle
    N = plan.n_field
    rng = np.random.default_rng(seed)
    blk = min(2048, N)
    blocks = [np.arange(0, blk), np.arange(N // 2, min(N, N // 2 + blk)), np.arange(N - blk, N)]
    rows = np.unique(np.concatenate([rng.choice(N, min(N, 5000), replace=False), *blocks]))
    rows = rows[(rows >= 0) & (rows < N)]
    er, ur = dense_materials(er_s)
    Eo, Bo, n_tets = oracle.rows_csr(field, er, ur, rows)
    ip, ix, Ev, Bv = plan.rows_host(rows, E, B)
    exact = bool(np.array_equal(ip, Eo.indptr) and np.array_equal(ix, Eo.indices)
                 and np.array_equal(ip, Bo.indptr) and np.array_equal(ix, Bo.indices))
    worst = {}
    for name, v, R in (("E", Ev, Eo), ("B", Bv, Bo)):
        rowmax = np.maximum.reduceat(np.abs(R.data), R.indptr[:-1])
        worst[name] = float(np.max(np.abs(v - R.data) / np.repeat(rowmax, np.diff(R.indptr)))) if exact else None
    return {"rows": int(len(rows)), "tets": int(n_tets), "pattern_exact": exact, "max_rel_E": worst["E"],
            "max_rel_B": worst["B"], "tol": 1e-12,
            "sample": "5000 random rows + 2048-row blocks at the start, middle and end of the DOF numbering"}


def run_topology(m, n, dev):
    """Mesh topology + DOF map of the same mesh: GPU sort build vs the NumPy host build.

    ``gpu_s``: host arrays in, host int64 arrays out (copies included);
    ``gpu_device_s``: device-resident tets / nodes in, device arrays out."""
    import torch
    from emerge_gb300.mesh import TetMesh
    from emerge_gb300.topology import build_topology
    build_topology(m.nodes, m.tets[:, :6000], dev)          # warm-up (library, sort temp sizes)
    nodes_d = torch.as_tensor(m.nodes, device=dev)
    tets_d = torch.as_tensor(m.tets.astype(np.int32), device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    build_topology(nodes_d, tets_d, dev, keep_on_device=True)
    torch.cuda.synchronize()
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    d = build_topology(m.nodes, m.tets, dev)
    t_gpu = time.perf_counter() - t0
    t0 = time.perf_counter()
    h = TetMesh(m.nodes, m.tets)
    t_host = time.perf_counter() - t0
    same = all(np.array_equal(getattr(h, k), d[k]) for k in ("edges", "tris", "tet_to_edge", "tet_to_tri",
                                                             "tri_to_edge", "tri_to_tet", "edge_lengths"))
    return {"workload": f"{n}^3 Kuhn cube: {m.n_tets} tets -> {h.n_edges} edges, {h.n_tris} faces",
            "gpu_device_s": round(t_dev, 4), "gpu_s": round(t_gpu, 4), "host_numpy_s": round(t_host, 3),
            "identical_to_host": bool(same)}


def _median_event_ms(fn, reps: int = 5, warm: int = 2) -> float:
    """Median CUDA-event time (ms) of fn() on the current stream."""
    import torch
    for _ in range(warm):
        fn()
    st = torch.cuda.current_stream()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(st)
        fn()
        b.record(st)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def sweep_rooflines(sw, freqs, n_anchor: int, chunk: int) -> dict:
    """HBM rooflines of the sweep's two memory-bound operators, timed alone with CUDA events
    on one chunk of the sweep's columns (c frequencies x 2 ports):

      spmv       — ``emg_spmv`` (kernel k_spmv / k_spmv_w): Y = A(k_c) X for every column,
                   A stored [nnz_r][c] complex128.  Algorithmic bytes per launch:
                   16 nnz_r c (matrix values, each read once) + 4 nnz_r (column indices)
                   + 8 (n+1) (row pointers) + 2 x 16 n 2c (X read, Y written).
      slab_apply — ``emg_slab_apply``: every column through its anchor's complex-FP32 slab
                   factor (forward and backward block sweep).  Algorithmic bytes: each used
                   factor's dense slab inverses read twice (2 x 8 sum w_i^2 per factor) +
                   4 x 16 n 2c (the right-hand side read, the result written, the forward
                   sweep's intermediate written and read back).
    """
    import torch
    peak, kind = peaks()
    c = max(1, min(len(freqs), chunk))
    fr = np.asarray(freqs[:c], dtype=float)
    k0, gam, _ = sw._coeffs(fr)
    A = sw.sys.form(sw.E, sw.B, k0 ** 2, sw.P, gam)
    n, nnz = sw.sys.n, sw.sys.nnz
    npo = len(sw.ports)
    gen = torch.Generator(device="cuda").manual_seed(0)
    X = torch.randn((n, c * npo), dtype=torch.complex128, device="cuda", generator=gen)
    cm = torch.arange(c, dtype=torch.int32, device="cuda").repeat_interleave(npo)
    ms = _median_event_ms(lambda: sw.sys.spmv(A, X, cm))
    b_spmv = 16 * nnz * c + 4 * nnz + 8 * (n + 1) + 2 * 16 * n * c * npo
    anchors = sw.default_anchors(freqs, n_anchor)
    sw.factor_anchors(anchors, "fp32")
    near = np.argmin(np.abs(fr[:, None] - anchors[None, :]), axis=1)
    cfac = np.repeat(near, npo)
    sl = sw.slab()
    off, _ = sl.levels()
    w = np.diff(off)
    ms_a = _median_event_ms(lambda: sl.apply(X, cfac))
    b_apply = 2 * 8 * int(np.sum(w * w)) * len(np.unique(near)) + 4 * 16 * n * c * npo
    del A, X
    torch.cuda.empty_cache()
    cols = c * npo
    f_spmv = 8 * nnz * cols                          # complex FP64 multiply-add = 8 flops
    f_apply = 2 * 8 * int(np.sum(w * w)) * cols      # two sweeps of complex FP32 multiply-adds
    sp = {"ms": round(ms, 4), "algorithmic_bytes": int(b_spmv), "achieved": b_spmv / ms / 1e6, "peak": peak,
          "unit": "GB/s", "frac": b_spmv / ms / 1e6 / peak,
          "compute": {"pipe": "fp64", "flops": int(f_spmv), "achieved_tflops": f_spmv / ms / 1e9,
                      "peak_tflops": FP64_TFLOPS, "frac": f_spmv / ms / 1e9 / FP64_TFLOPS}}
    ap = {"ms": round(ms_a, 4), "algorithmic_bytes": int(b_apply), "achieved": b_apply / ms_a / 1e6, "peak": peak,
          "unit": "GB/s", "frac": b_apply / ms_a / 1e6 / peak,
          "compute": {"pipe": "fp32", "flops": int(f_apply), "achieved_tflops": f_apply / ms_a / 1e9,
                      "peak_tflops": FP32_TFLOPS, "frac": f_apply / ms_a / 1e9 / FP32_TFLOPS},
          "factors_used": int(len(np.unique(near))), "sum_w2": int(np.sum(w * w)), "slabs": int(len(w))}
    for d in (sp, ap):
        d["bound"] = "compute (" + d["compute"]["pipe"] + ")" if d["compute"]["frac"] > d["frac"] else "hbm"
    return {"columns": int(cols), "matrices": int(c), "n": int(n), "nnz_r": int(nnz), "peak_source": kind,
            "spmv": sp, "slab_apply": ap}


def factor_rate(sl, n_factors: int, seconds: float) -> dict:
    off, _ = sl.levels()
    w = np.diff(off).astype(np.float64)
    flops = 8.0 * float(np.sum(w ** 3)) * n_factors
    tf = flops / seconds / 1e12 if seconds > 0 else None
    return {"gj_flops": flops, "achieved_tflops": tf, "fp32_cuda_core_tflops": FP32_TFLOPS,
            "frac_of_fp32_cuda_core": tf / FP32_TFLOPS if tf else None,
            "note": "wall time of the whole factorization (pivot-tile chain, panels, Schur complements)"}


def run_sweep(args):
    """Iris-filter sweep: batched + mixed-precision + warm-started vs the plain FP64 GPU solve.

    freq-pts/s = points / wall time of the solve phase (volume and port matrices
    assembled before; every method forms A(k) itself and pays its own factorizations).
      plain  — one frequency at a time: slab factorization of A(k) in complex FP64 +
               FGMRES (a direct solve: 1-2 iterations), both ports together; timed
               on ``--sweep-plain`` points spread over the band, rate extrapolated.
      fast   — all points: FP32 slab factors at ``--sweep-anchors`` anchor
               frequencies (one batched factorization), ``--sweep-train`` points spread
               over the band solved by batched FGMRES, the minimal-residual projection
               onto their span as every other point's initial guess, then batched
               FGMRES on those columns to the same FP64 residual tolerance.
      mlp    — the same with the BF16 tensor-core MLP (trained on ``--sweep-mlp-train``
               points' own basis coefficients) supplying the initial guesses instead of
               the projection.
      mlp_minres — the network trained instead on the reduced system's minimal-residual
               coefficients at 256 frequencies, from the projection's training points.
      cold   — the same anchored batched FGMRES from zero initial guesses.
      plain_fp32_factor — plain with a complex-FP32 factorization per point and FP64
               FGMRES to the same tolerance (the per-point method without the FP64 rate).
    max|dS| compares each with plain on the plain points (spread points plus the two
    strongest passband peaks), and with an independent per-point check on 16 points
    that include the five passband peaks (``check``).  ``roofline``: the HBM rooflines
    of the SpMV and of the slab-factor apply (see sweep_rooflines).  Also reported: the
    ILU(0)-GMRES plain method on one point with capped iterations, and SciPy's
    SuperLU (the reference's default direct solver) per point on the host cores.
    """
    import torch
    from emerge_gb300.freq import Assembler
    from emerge_gb300.geometry import iris_filter
    from emerge_gb300.solver import FrequencySweep
    p = iris_filter(args.sweep_h, hy=args.sweep_hy)
    asm = Assembler()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sw = FrequencySweep(asm, p.field, p.er, p.ur, p.bcs)
    sl = sw.slab()
    torch.cuda.synchronize()
    setup = time.perf_counter() - t0
    nf = args.sweep_points
    freqs = np.linspace(8e9, 12e9, nf)
    idx = np.unique(np.linspace(0, nf - 1, args.sweep_plain + 2).astype(int)[1:-1])
    # points per batched solve: every column at once unless the Krylov basis (V and Z,
    # restart+1 and restart vectors of n x 2 columns per point, complex128) and the
    # stored A(k) would pass ~80 GB
    per_point = 16 * (2 * sw.sys.n * (2 * args.sweep_restart + 3) + sw.sys.nnz)
    chunk = args.sweep_chunk or max(1, min(nf, int(80e9 // per_point)))
    out = {"workload": f"{p.name}: N={p.field.n_field} DOFs ({sw.sys.n} after PEC), {nf} points 8-12 GHz x 2 ports",
           "metric": "sweep freq-pts/s", "tol": args.sweep_tol, "setup_s": round(setup, 2),
           "slabs": sl.info()["slabs"], "max_slab_width": sl.info()["max_width"], "chunk_points": chunk}
    # the slab products' layout, tuned once per mesh and column pattern (not timed)
    out["autotune"] = sw.autotune(freqs, n_anchor=args.sweep_anchors, chunk=chunk)
    out["autotune"]["seconds"] = round(out["autotune"]["seconds"], 2)
    out["roofline"] = sweep_rooflines(sw, freqs, args.sweep_anchors, chunk)
    if args.sweep_rooflines_only:
        return out
    kw = dict(precision="fp32", tol=args.sweep_tol, restart=args.sweep_restart, chunk=chunk,
              refine=args.sweep_refine, inner=args.sweep_inner)
    with ClockSampler(0) as clk:
        # warm-up of every code path on a tiny sweep (graph capture, cuBLAS/cuSOLVER handles)
        # (the basis sizes of the timed runs, on every tenth frequency)
        for guess, ntr in (("projection", args.sweep_train), ("mlp", args.sweep_mlp_train)):
            sw.run_warm(freqs[::10], n_train=min(ntr, len(freqs[::10]) - 1), solver="anchored", n_anchor=1,
                        precision="fp32", guess=guess, tol=args.sweep_tol, mlp_steps=50)
        # every variant pays its own anchor factorization (the factors are cached per key)
        sw._slab_key = None
        fast = sw.run_warm(freqs, n_train=min(args.sweep_train, nf), solver="anchored", n_anchor=args.sweep_anchors,
                           guess="projection", **kw)
        sw._slab_key = None
        mlp = sw.run_warm(freqs, n_train=min(args.sweep_mlp_train, nf), solver="anchored",
                          n_anchor=args.sweep_anchors, guess="mlp", mlp_steps=args.sweep_mlp_steps, **kw)
        sw._slab_key = None
        mlp_mr = sw.run_warm(freqs, n_train=min(args.sweep_train, nf), solver="anchored",
                             n_anchor=args.sweep_anchors, guess="mlp", mlp_steps=args.sweep_mlp_minres_steps,
                             mlp_target="minres", **kw)
        sw._slab_key = None
        cold = sw.run_anchored(freqs, n_anchor=args.sweep_anchors, **kw)
        # the passband peaks of |S21| (resonances, where the sweep is hardest): the largest
        # local maxima of the fast sweep's |S21|
        s21 = np.abs(fast.S[:, 1, 0])
        loc = np.flatnonzero((s21[1:-1] > s21[:-2]) & (s21[1:-1] >= s21[2:])) + 1
        peaks_i = np.sort(loc[np.argsort(s21[loc])[::-1][:5]])
        # the plain FP64 solver on spread points plus the two strongest peaks
        idx = np.unique(np.concatenate([idx, peaks_i[np.argsort(s21[peaks_i])[::-1][:args.sweep_plain_peaks]]]))
        plain = sw.run(freqs[idx], method="plain", precond="slab64", tol=args.sweep_tol)
        # the same per-point method with a complex-FP32 factorization and FP64 FGMRES: the
        # per-point baseline without GB300's FP64 rate in it
        plain32 = sw.run(freqs[idx], method="plain", precond="slab32", tol=args.sweep_tol)
    # independent check on 16 points (the peaks + spread points): every column
    # preconditioned by a factorization at its own frequency, FGMRES to a 1e-12 FP64
    # residual (no warm start, no shared anchors), untimed
    spread = np.linspace(0, nf - 1, max(2, args.sweep_check - len(peaks_i)) + 2).astype(int)[1:-1]
    chk = np.unique(np.concatenate([peaks_i, spread]))
    sw._slab_key = None
    check = sw.run_anchored(freqs[chk], anchors=freqs[chk], precision="fp32", tol=1e-12,
                            restart=args.sweep_restart)
    sw._slab_key = None
    v_fast = nf / fast.seconds
    v_plain = len(idx) / plain.seconds
    pred = mlp.info["final_index"]
    common = np.flatnonzero(np.isin(chk, idx))
    out.update({
        "fast": v_fast, "plain": v_plain, "ratio": v_fast / v_plain,
        "max_abs_dS_vs_plain": float(np.max(np.abs(fast.S[idx] - plain.S))),
        "plain_points_GHz": [round(float(f) / 1e9, 4) for f in freqs[idx]],
        "check": {"points": int(len(chk)), "points_GHz": [round(float(f) / 1e9, 4) for f in freqs[chk]],
                  "passband_peaks_GHz": [round(float(f) / 1e9, 4) for f in freqs[peaks_i]],
                  "S21_dB_at_peaks": [round(float(20 * np.log10(s21[i] + 1e-300)), 3) for i in peaks_i],
                  "method": "per point: complex-FP32 slab factor of A(k) at that frequency, FP64 FGMRES to 1e-12",
                  "max_residual": float(check.residuals.max()),
                  "max_abs_dS_fast": float(np.max(np.abs(fast.S[chk] - check.S))),
                  "max_abs_dS_mlp": float(np.max(np.abs(mlp.S[chk] - check.S))),
                  "max_abs_dS_cold": float(np.max(np.abs(cold.S[chk] - check.S))),
                  "max_abs_dS_plain_vs_check": float(np.max(np.abs(plain.S[np.searchsorted(idx, chk[common])]
                                                                   - check.S[common]))) if common.size else None},
        "max_residual_fast": float(fast.residuals.max()), "max_residual_plain": float(plain.residuals.max()),
        "fast_seconds": round(fast.seconds, 3), "plain_seconds_per_point": round(plain.seconds / len(idx), 3),
        "plain_points_timed": int(len(idx)), "anchors": args.sweep_anchors, "precision_inner": "complex fp32",
        "fast_guess": "projection", "factor_seconds": round(float(fast.info.get("factor_seconds", 0.0)), 3),
        # Gauss-Jordan flops of the anchors' factorization (8 sum w^3 per factor, complex
        # multiply-add = 8 flops) over its wall time, against the FP32 CUDA-core rate
        "factor_rate": factor_rate(sl, args.sweep_anchors, float(fast.info.get("factor_seconds", 0.0))),
        "train_points": int(fast.info["train_points"]), "train_seconds": round(fast.info["train_seconds"], 3),
        "guess_seconds": round(fast.info["guess_seconds"], 3), "final_seconds": round(fast.info["final_seconds"], 3),
        "iterations_fast_mean": float(fast.iterations.mean()), "iterations_fast_max": int(fast.iterations.max()),
        "iterations_fast_predicted_mean": fast.info["final_iterations_mean"],
        "mlp": {"pts_per_s": nf / mlp.seconds, "seconds": round(mlp.seconds, 3),
                "train_points": int(mlp.info["train_points"]), "train_seconds": round(mlp.info["train_seconds"], 3),
                "mlp_seconds": round(mlp.info["guess_seconds"], 3), "mlp_loss": mlp.info["mlp_loss"],
                "final_seconds": round(mlp.info["final_seconds"], 3),
                # iterations on the points the network predicts (all but its training points)
                "iterations_predicted_mean": mlp.info["final_iterations_mean"],
                "iterations_cold_same_points_mean": float(cold.iterations[pred].mean()),
                "max_abs_dS_vs_plain": float(np.max(np.abs(mlp.S[idx] - plain.S)))},
        # the network trained on the reduced system's minimal-residual coefficients at
        # 256 frequencies, from the projection's 12 training points
        "mlp_minres": {"pts_per_s": nf / mlp_mr.seconds, "seconds": round(mlp_mr.seconds, 3),
                       "train_points": int(mlp_mr.info["train_points"]),
                       "train_seconds": round(mlp_mr.info["train_seconds"], 3),
                       "mlp_seconds": round(mlp_mr.info["guess_seconds"], 3), "mlp_loss": mlp_mr.info["mlp_loss"],
                       "final_seconds": round(mlp_mr.info["final_seconds"], 3),
                       "iterations_predicted_mean": mlp_mr.info["final_iterations_mean"],
                       "iterations_cold_same_points_mean": float(cold.iterations[mlp_mr.info["final_index"]].mean()),
                       "max_abs_dS_check": float(np.max(np.abs(mlp_mr.S[chk] - check.S)))},
        "plain_fp32_factor": {"pts_per_s": len(idx) / plain32.seconds,
                              "seconds_per_point": round(plain32.seconds / len(idx), 3),
                              "iterations_mean": float(plain32.iterations.mean()),
                              "max_residual": float(plain32.residuals.max()),
                              "max_abs_dS_vs_plain": float(np.max(np.abs(plain32.S - plain.S))),
                              "fast_ratio": v_fast / (len(idx) / plain32.seconds)},
        "cold": {"pts_per_s": nf / cold.seconds, "seconds": round(cold.seconds, 3),
                 "iterations_mean": float(cold.iterations.mean()), "iterations_max": int(cold.iterations.max()),
                 "max_abs_dS_vs_fast": float(np.max(np.abs(cold.S - fast.S)))},
        "inner": args.sweep_inner, "refine": args.sweep_refine,
        "refinement_steps": int(fast.info.get("refinement_steps", 0)),
        "iterations_plain_mean": float(plain.iterations.mean()),
        "S21_db_samples": [round(float(20 * np.log10(abs(v) + 1e-300)), 2) for v in fast.S[::max(1, nf // 8), 1, 0]],
        "clocks": clk.summary(),
    })
    if args.sweep_ilu_iters > 0:
        ilu = sw.run(freqs[idx[:1]], method="plain", precond="ilu0", tol=args.sweep_tol, max_iter=args.sweep_ilu_iters)
        out["ilu0_plain_probe"] = {"points": 1, "max_iter": args.sweep_ilu_iters,
                                   "iterations": int(ilu.iterations.max()), "residual": float(ilu.residuals.max()),
                                   "seconds": round(ilu.seconds, 2),
                                   "converged": bool(ilu.residuals.max() <= args.sweep_tol * 10)}
    if args.sweep_cpu > 0:
        out["cpu_superlu"] = cpu_superlu(sw, freqs[idx[:args.sweep_cpu]], plain)
    return out


# FP32 operations of one (source, direction) term of k_ff_sum (multiply and add counted
# separately, sincosf excluded): phase 5, r x (n x H) 18, n x E - Z0 (...) 12,
# rotation by G 18, accumulation of r x ie 24
FF_FLOPS_PER_PAIR = 77
def run_farfield(dev):
    """Stratton-Chu far field: 20k surface sources x 181 x 360 directions on the GPU,
    against the NumPy restatement on a 300-direction sample of the same sources."""
    import types
    import torch
    from emerge_gb300.farfield import stratton_chu
    rng = np.random.default_rng(3)
    ns, nt = 20000, 30000
    mesh = types.SimpleNamespace(n_tris=nt, tri_to_edge=rng.integers(0, ns, (3, nt)),
                                 normals=rng.normal(size=(3, nt)), areas=rng.uniform(1e-6, 2e-6, nt),
                                 edge_centers=rng.uniform(-0.1, 0.1, (3, ns)))
    E = rng.normal(size=(3, ns)) + 1j * rng.normal(size=(3, ns))
    H = (rng.normal(size=(3, ns)) + 1j * rng.normal(size=(3, ns))) / 377
    th, ph = np.meshgrid(np.linspace(-np.pi / 2, np.pi / 2, 181), np.linspace(0, 2 * np.pi, 360, endpoint=False),
                         indexing="ij")
    th, ph = th.ravel(), ph.ravel()
    k0 = 2 * np.pi * 10e9 / 299792458
    import ctypes
    from emerge_gb300 import _lib
    from emerge_gb300.farfield import surface_weights
    t0 = time.perf_counter()
    Eg, _ = stratton_chu(E, H, mesh, th, ph, k0, dev)                       # also the warm-up
    t_call = time.perf_counter() - t0
    # the device entry point alone, inputs resident: the transform's own time
    d = {k: torch.as_tensor(np.ascontiguousarray(v), device=dev) for k, v in
         (("E", E.astype(np.complex64)), ("H", H.astype(np.complex64)),
          ("v", mesh.edge_centers.astype(np.float32)), ("w", surface_weights(mesh)),
          ("th", th.astype(np.float32)), ("ph", ph.astype(np.float32)))}
    Eo_d = torch.empty((3, th.size), dtype=torch.complex128, device=dev)
    Ho_d = torch.empty_like(Eo_d)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())                                          # noqa: E731
    reps = 5
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        _lib.call("emg_stratton_chu", ns, vp(d["E"]), vp(d["H"]), vp(d["v"]), vp(d["w"]), th.size, vp(d["th"]),
                  vp(d["ph"]), ctypes.c_float(k0), vp(Eo_d), vp(Ho_d),
                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    t_gpu = (time.perf_counter() - t0) / reps
    pairs = ns * th.size
    out = {"workload": f"{ns} sources x {th.size} directions (181 x 360), 10 GHz",
           "device_call_s": round(t_gpu, 5), "host_call_s": round(t_call, 4), "pairs_per_s": pairs / t_gpu,
           "compute": {"bound": "fp32", "flops_per_pair": FF_FLOPS_PER_PAIR, "peak_tflops": FP32_TFLOPS,
                       "achieved_tflops": pairs * FF_FLOPS_PER_PAIR / t_gpu / 1e12,
                       "frac": pairs * FF_FLOPS_PER_PAIR / t_gpu / 1e12 / FP32_TFLOPS,
                       "note": "emg_stratton_chu wall time with device-resident inputs (its scratch "
                               "allocation and final synchronisation included); sincosf not counted"}}
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from oracle import farfield_oracle as fo
    wns = surface_weights(mesh)
    sel = np.arange(0, th.size, th.size // 300)[:300]
    t0 = time.perf_counter()
    Eo, _ = fo.stratton_chu_ff(E, H, mesh.edge_centers, wns, th[sel], ph[sel], k0)
    t_cpu = time.perf_counter() - t0
    out["cpu_baseline"] = {"pairs_per_s": ns * sel.size / t_cpu, "kind": "port", "cores": os.cpu_count(),
                           "sample": f"{sel.size} of the directions, NumPy FP64 restatement"}
    out["max_rel_diff_vs_port"] = float(np.abs(Eg[:, sel] - Eo).max() / np.abs(Eo).max())
    return out


def run_eigen(args):
    """Cavity eigenmodes: ``--eigen`` instances of the seeded 64-cavity batch (sides
    U[15,40] mm, dielectric cylinder r U[2,6] mm, eps U[2,30], h = 2.2 mm; the smallest,
    or with ``--eigen-select spread`` instances spread over the size range), 10 lowest
    nonzero modes each, one instance after another.  The first instance is
    checked against SciPy ARPACK (eigs, shift-invert, the reference's method) on the
    host: max relative eigenvalue error."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla
    import torch
    from emerge_gb300.eigen import CavityEigen, box_sigma
    from emerge_gb300.freq import Assembler
    from emerge_gb300.geometry import cavity_set
    ps = cavity_set(64, seed=4, h=args.eigen_h)
    by_size = sorted(range(64), key=lambda i: ps[i].field.n_field)
    if args.eigen_select == "spread":   # evenly spaced size ranks, the smallest and the largest included
        ranks = np.unique(np.round(np.linspace(0, 63, max(1, args.eigen))).astype(int))
        order = [by_size[r] for r in ranks]
        which = f"{len(order)} of 64 seeded PEC cavities at evenly spaced size ranks (smallest to largest)"
    else:
        order = by_size[: args.eigen]
        which = f"{len(order)} smallest of 64 seeded PEC cavities"
    asm = Assembler()
    out = {"workload": f"{which} with dielectric cylinders, h={args.eigen_h}",
           "modes": args.eigen_modes, "instances": []}
    total = 0.0
    err = None
    # warm-up on a small cavity (graph capture, solver handles): the timed instances
    # are then the steady state of a batch
    from emerge_gb300.geometry import dielectric_cavity
    pw = dielectric_cavity(12e-3, 10e-3, 8e-3, 2e-3, 6.0, 2e-3)
    cw = CavityEigen(asm, pw.field, pw.er, pw.ur, pw.bcs)
    cw.solve(min(6, args.eigen_modes), sigma=box_sigma(np.array([12e-3, 10e-3, 8e-3]), 6.0), which="LR", tol=1e-10)
    del cw
    asm._dev = None
    with ClockSampler(0) as clk:
        for k, i in enumerate(order):
            p = ps[i]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ce = CavityEigen(asm, p.field, p.er, p.ur, p.bcs)
            nodes = np.asarray(p.mesh.nodes)
            dims = nodes.max(axis=1) - nodes.min(axis=1)
            sigma = box_sigma(dims, float(np.max(np.abs(p.er[0, 0]))))
            r = ce.solve(args.eigen_modes, sigma=sigma, which="LR", tol=1e-10)
            torch.cuda.synchronize()
            secs = time.perf_counter() - t0
            total += secs
            out["instances"].append({"n": int(ce.sys.n), "seconds": round(secs, 2), "max_residual": float(r.residuals.max()),
                                     "restarts": r.info["restarts"], "solves": r.info["solves"],
                                     "slabs": r.info["slabs"], "max_slab_width": r.info["max_width"],
                                     "f_GHz": [round(float(f) / 1e9, 5) for f in r.frequencies[:3]]})
            if k == 0 and args.eigen_check:
                ptr, ind = ce.sys.pattern()
                n = ce.sys.n
                E = sps.csc_matrix(sps.csr_matrix((ce.Er[:, 0].cpu().numpy(), ind, ptr), shape=(n, n)))
                B = sps.csc_matrix(sps.csr_matrix((ce.Br[:, 0].cpu().numpy(), ind, ptr), shape=(n, n)))
                t1 = time.perf_counter()
                ref = np.sort(spla.eigs(E, k=args.eigen_modes, M=B, sigma=sigma, which="LR", tol=1e-13)[0].real)
                out["arpack_seconds"] = round(time.perf_counter() - t1, 2)
                err = float(np.max(np.abs(np.sort(r.eigenvalues.real) - ref) / ref))
            del ce
            asm._dev = None
    out.update({"seconds_total": round(total, 2), "instances_per_s": len(order) / total,
                "max_rel_eig_error_vs_arpack": err, "clocks": clk.summary()})
    return out


def cpu_superlu(sw, freqs, plain):
    """SciPy SuperLU (the reference's SolverSuperLU) on the host: per point factor + 2-port solve."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla
    import torch
    sysr = sw.sys
    n = sysr.n
    k0, gam, beta = sw._coeffs(freqs)
    A = sysr.form(sw.E, sw.B, k0 ** 2, sw.P, gam).cpu().numpy()            # (nnz_r, nf)
    rhs = sw._rhs(beta).cpu().numpy()                                       # (n, nf*np)
    ptr_t, ind_t = sysr.pattern()
    npo = len(sw.ports)
    t0 = time.perf_counter()
    err = 0.0
    from scipy.sparse.csgraph import reverse_cuthill_mckee
    for f in range(len(freqs)):
        # SolveRoutine with ReverseCuthillMckee + SolverSuperLU (fem/solver.py:135-151, 243-275)
        M = sps.csr_matrix((A[:, f], ind_t, ptr_t), shape=(n, n))
        perm = reverse_cuthill_mckee(M)
        Ms = sps.csc_matrix(M[perm, :][:, perm])
        lu = spla.splu(Ms, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.01, options=dict(SymmetricMode=True))
        Xs = lu.solve(rhs[perm, f * npo:(f + 1) * npo])
        X = np.empty_like(Xs)
        X[perm] = Xs
        S = sw._sparams(torch.as_tensor(X, device=sw.device), 1, beta[:, f:f + 1], k0[f:f + 1])
        err = max(err, float(np.max(np.abs(S[0] - plain.S[f]))))
    secs = time.perf_counter() - t0
    return {"value": len(freqs) / secs, "unit": "freq-pts/s", "points": len(freqs), "cores": os.cpu_count(),
            "kind": "reference", "seconds_per_point": round(secs / len(freqs), 2), "max_abs_dS_vs_gpu_plain": err,
            "sample": "scipy.sparse.linalg.splu + solve of the same restricted A(k), 2 ports, per point"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--n", type=int, default=80, help="hexes per cube side (80 -> 3.07M tets)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=200_000, help="tets in the bounded CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-sweep", action="store_true", help="skip the frequency-sweep measurement")
    ap.add_argument("--sweep-h", type=float, default=2e-3, help="iris-filter mesh size across the guide (m)")
    ap.add_argument("--sweep-hy", type=float, default=1.3e-3,
                    help="iris-filter grid spacing along the guide (m): 1.3 mm gives ~3e5 DOFs at h = 2 mm")
    ap.add_argument("--sweep-points", type=int, default=401)
    ap.add_argument("--sweep-train", type=int, default=12, help="points solved first; their span gives the guesses")
    ap.add_argument("--sweep-mlp-train", type=int, default=32, help="training points of the MLP variant")
    ap.add_argument("--sweep-anchors", type=int, default=2)
    ap.add_argument("--sweep-restart", type=int, default=40)
    ap.add_argument("--sweep-chunk", type=int, default=0, help="points per batched solve (0: as many as fit ~80 GB)")
    ap.add_argument("--sweep-mlp-steps", type=int, default=300)
    ap.add_argument("--sweep-mlp-minres-steps", type=int, default=1500,
                    help="training steps of the network on minimal-residual targets")
    ap.add_argument("--sweep-inner", default="fp64", choices=["fp32", "fp64"],
                    help="precision of the Krylov vectors of the fast sweep (its factors are FP32 either way)")
    ap.add_argument("--sweep-refine", type=int, default=0, help="Newton-Schulz step on the FP32 slab inverses")
    ap.add_argument("--sweep-plain", type=int, default=2, help="spread points timed with the plain FP64 solver")
    ap.add_argument("--sweep-plain-peaks", type=int, default=2, help="passband peaks added to the plain points")
    ap.add_argument("--sweep-check", type=int, default=16, help="points of the independent S-parameter check")
    ap.add_argument("--sweep-rooflines-only", action="store_true",
                    help="with --sweep-only: build the iris sweep and measure only the SpMV / slab-apply rooflines")
    ap.add_argument("--sweep-ilu-iters", type=int, default=1000)
    ap.add_argument("--sweep-cpu", type=int, default=1, help="points solved by SciPy SuperLU on the host")
    ap.add_argument("--sweep-tol", type=float, default=1e-8)
    ap.add_argument("--sweep-only", action="store_true", help="print only the sweep measurement")
    ap.add_argument("--eigen", type=int, default=2, help="cavity eigen instances (0: skip)")
    ap.add_argument("--eigen-h", type=float, default=2.2e-3)
    ap.add_argument("--eigen-modes", type=int, default=10)
    ap.add_argument("--eigen-check", type=int, default=1, help="ARPACK check of the first instance")
    ap.add_argument("--eigen-select", default="smallest", choices=["smallest", "spread"],
                    help="the smallest instances, or instances spread over the size range")
    ap.add_argument("--eigen-only", action="store_true", help="print only the eigen measurement")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.sweep_only:
        if rank == 0:
            print(json.dumps(run_sweep(args)))
    elif args.eigen_only:
        if rank == 0:
            print(json.dumps(run_eigen(args)))
    else:
        run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Benchmark of the two-site DMRG sweep (the TenNetLib.jl hot path) on one GB300.

Workload (the U(1) Heisenberg configuration of the metric): open S=1/2 Heisenberg chain,
N = 100, total S^z = 0, MPO bond dimension 5, Neel start, maxdim ramp 64 -> 1024, cutoff
1e-12, Lanczos krylovdim 5 / maxiter 2 (eig_solver defaults).  The ramp 64, 128, 256, 512,
1024 (two sweeps each) prepares the state untimed; a step is then one full two-site sweep
(left-to-right and right-to-left, 2 (N - 1) bond updates) at maxdim 1024.  The bond
dimension is limited by the cutoff (about 180 after convergence).

The JSON line reports seconds per sweep (device time from CUDA events inside the library),
the H_eff contraction throughput, the grouped-GEMM roofline, the end-to-end time through
the C ABI with host buffers, and the CPU oracle timed on the host cores.

Multi-GPU: sweeps are sequential in the bond position, so N GPUs run N independent
replicas (no collective on the data path); the value is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sweep s & H_eff TFLOP/s, split-prec vs FP64 GPU at |ΔE/E|≤1e-10"
N_SITES = 100
RAMP = [64, 128, 256, 512, 1024]
MAXDIM = 1024
CUTOFF = 1e-12
KRYLOVDIM = 5
MAXITER = 2
FP64_PEAK_NOMINAL_TFLOPS = 1.25  # GB300 FP64 (no measured FP64 peak on this machine)
# GB300 FP32 on the CUDA cores: 152 SMs x 128 lanes x 2 flops x 2.07 GHz (nominal)
FP32_PEAK_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "fallback": True}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"tn_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def heisenberg(tn, ctx):
    W, delta, pq = tn.models.mpo_from_terms(N_SITES, tn.models.heisenberg_chain_terms(N_SITES))
    return tn.MPO(W, delta, pq, ctx), pq


def sweep_kwargs(maxdim):
    return dict(maxdim=maxdim, cutoff=CUTOFF, solver_krylovdim=KRYLOVDIM, solver_maxiter=MAXITER,
                outputlevel=0)


def download_state(psi):
    """Dense host copy of an engine MPS: (tensors, link charge arrays)."""
    tensors = [psi.site(i) for i in range(psi.N)]
    links = [psi.link_charges(i) for i in range(psi.N + 1)]
    return tensors, links


def download_blocks(psi):
    """Block-sparse host copy of an engine MPS (the charge blocks only, as an ITensors QN MPS
    stores them): (per-site block arrays, link charge arrays)."""
    blocks = [psi.site_blocks(i) for i in range(psi.N)]
    links = [psi.link_charges(i) for i in range(psi.N + 1)]
    return blocks, links


# ------------------------------------------------------------------------------------
# CPU oracle legs (timed as the CPU baseline / reference arm)
# ------------------------------------------------------------------------------------

def oracle_env_from(tensors, links):
    import numpy as np
    from oracle import tn_oracle as O
    H = O.heisenberg_mpo(N_SITES)
    psi = O.MPS([np.asarray(t) for t in tensors], [np.asarray(q, dtype=np.int64) for q in links],
                O.SPIN_HALF_Q.copy(), center=0)
    return O, O.StateEnvs(psi, H)


def oracle_halfsweep(O, env, direction):
    """One half sweep (N - 1 bond updates) of the oracle; returns the last energy."""
    N = env.N
    bonds = range(N - 1) if direction == "left" else range(N - 2, -1, -1)
    e = None
    for b in bonds:
        e, _, _ = O.update_two_site(env, b, direction, MAXDIM, 1, CUTOFF, KRYLOVDIM, MAXITER, 1e-14)
    return e


def cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_baseline_from(tensors, links):
    """Time one full oracle sweep from the GPU-prepared state on the host cores; also return
    the oracle's energy and largest bond dimension after that sweep."""
    O, env = oracle_env_from(tensors, links)
    env.position(0, 2)  # right environments: setup, not timed
    t0 = time.perf_counter()
    oracle_halfsweep(O, env, "left")
    e = oracle_halfsweep(O, env, "right")
    dt = time.perf_counter() - t0
    return {"value": dt, "unit": "s/sweep", "cores": cores(), "kind": "port", "dense": True,
            "energy": e, "maxlinkdim": int(env.psi.maxlinkdim()),
            "sample": f"one full two-site sweep ({2 * (N_SITES - 1)} bond updates) of the numpy "
                      "FP64 oracle (dense tensors with charge labels, not block-sparse; OpenBLAS "
                      "threads = all host cores) from the same converged chi~180 state"}


def run_reference(args, world, rank, pg):
    """--impl reference: the oracle port on the host cores (the reference is Julia and
    cannot run here).  Each step is one full two-site sweep at maxdim 1024."""
    if rank != 0:
        return
    import numpy as np
    from oracle import tn_oracle as O
    H = O.heisenberg_mpo(N_SITES)
    psi = O.product_mps([0 if i % 2 == 0 else 1 for i in range(N_SITES)], O.SPIN_HALF_Q)
    env = O.StateEnvs(psi, H)
    sw = O.SweepData()
    for md in RAMP:  # prepare (not timed)
        O.fullsweep(env, sw, md, CUTOFF, 1, KRYLOVDIM, MAXITER, 1e-14)
    for _ in range(args.warmup):
        oracle_halfsweep(O, env, "left")
        oracle_halfsweep(O, env, "right")
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle_halfsweep(O, env, "left")
        oracle_halfsweep(O, env, "right")
        times.append(time.perf_counter() - t0)
    value = statistics.mean(times)
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s/sweep",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config(args),
        "cpu_baseline": {"value": value, "unit": "s/sweep", "cores": cores(), "kind": "port",
                         "dense": True,
                         "sample": "per step one full two-site sweep (198 bond updates) of the "
                                   "numpy FP64 oracle (dense tensors with charge labels, not "
                                   "block-sparse) from its own converged chi~180 state "
                                   "(TenNetLib.jl itself needs Julia + ITensors, absent here)"},
        "e2e": {"value": value, "unit": "s/sweep", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------------------------
# TTN leg: 32 transverse-field Ising instances on the 64-site binary tree
# ------------------------------------------------------------------------------------
TTN_SITES = 64
TTN_INSTANCES = 32
TTN_CHIS = [64, 128, 256]


def tfim_ground_energy(J, h):
    """Open TFIM ground energy by Jordan-Wigner: minus the sum of the singular values of
    the bidiagonal matrix (h_i on the diagonal, J_i above it)."""
    import numpy as np
    B = np.diag(np.asarray(h, dtype=float)) + np.diag(np.asarray(J, dtype=float), 1)
    return -float(np.linalg.svd(B, compute_uv=False).sum())


def run_ttn(tn, device, args, world):
    """One lockstep sweep of all instances (after one warm-up sweep); device time."""
    ctx = tn.Context(device, precision=args.precision, slices=args.slices)
    T = tn.ttn
    chis, psis, models, exact = [], [], [], []
    t0 = time.perf_counter()
    for i in range(args.ttn_instances):
        chi = TTN_CHIS[i % len(TTN_CHIS)]
        J, h = T.tfim_instance(TTN_SITES, 1000 + i)
        chis.append(chi)
        psis.append(T.default_randomTTN(TTN_SITES, chi, 2000 + i, ctx=ctx))
        models.append(T.CouplingModel(T.tfim_terms(J, h), TTN_SITES))
        exact.append(tfim_ground_energy(J, h))
    envs = T.StateEnvsTTN.batch(psis, models)
    prep = time.perf_counter() - t0
    path = T.default_sweeppath(TTN_SITES)
    sws = [T.SweepDataTTN() for _ in envs]
    kw = dict(maxdim=max(TTN_CHIS), outputlevel=0)
    T.fullsweep_batch_(envs, path, tn.eig_solver, sws, **kw)      # warm-up
    print(f"ttn_launches_before_timed={ctx.lib.tn_kernel_launches()}", file=sys.stderr,
          flush=True)
    t1 = time.perf_counter()
    T.fullsweep_batch_(envs, path, tn.eig_solver, sws, **kw)      # timed
    wall = time.perf_counter() - t1
    st = sws[0].stats[-1]
    dev_s = st["sweep_ms"] / 1e3
    rel = [abs(sw.energy[-1] - e) / abs(e) for sw, e in zip(sws, exact)]
    out = {
        "workload": f"tfim_binary_tree_64_sites_{args.ttn_instances}_instances_maxdim_64_128_256",
        "instances": args.ttn_instances, "maxdim_cycle": TTN_CHIS, "sweeps_before_timed": 1,
        "value": dev_s, "unit": "s/sweep (all instances, lockstep)",
        "wall_s": wall, "prepare_s": prep,
        "heff_tflops": st["heff_flops"] / max(st["heff_ms"], 1e-9) / 1e9,
        "heff_flops_per_sweep": st["heff_flops"],
        "time_share": {k: st[k] / max(st["sweep_ms"], 1e-9)
                       for k in ("heff_ms", "env_ms", "svd_ms", "lanczos_ms", "pack_ms")},
        "time_share_note": "svd_ms = QR isometry moves; env_ms = link-tensor moves",
        "matvecs": st["matvecs"], "gpu_launches": st["kernel_launches"],
        "krylov_hbm_gbs": st["krylov_bytes"] / max(st["lanczos_ms"], 1e-9) / 1e6,
        "qr_panel_s": st["qr_panel_ms"] / 1e3, "qr_gemm_s": st["qr_gemm_ms"] / 1e3,
        "max_rel_energy_error_vs_free_fermion_after_2_sweeps": max(rel),
        "median_rel_energy_error_after_2_sweeps": statistics.median(rel),
    }
    if world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = ttn_cpu_baseline()
    return out


def ttn_cpu_baseline():
    """The numpy oracle on a bounded sample: one sweep of instance 0 (maxdim 64)."""
    from oracle import ttn_oracle as O
    J, h = O.tfim_instance(TTN_SITES, 1000)
    se = O.StateEnvsTTN(O.random_ttn(TTN_SITES, TTN_CHIS[0], 2000), O.tfim_terms(J, h))
    g, _ = O.default_graph_sitenodes(TTN_SITES)
    sw = O.SweepDataTTN()
    t0 = time.perf_counter()
    O.fullsweep(se, O.default_sweeppath(TTN_SITES, g.keys()), sw, maxdim=TTN_CHIS[0])
    dt = time.perf_counter() - t0
    return {"value": dt, "unit": "s/sweep of one maxdim-64 instance", "cores": cores(),
            "kind": "port",
            "sample": "one sweep (124 node updates) of instance 0 (maxdim 64) by the numpy "
                      "FP64 TTN oracle; maxdim-128 and -256 instances cost about 8x and 100x "
                      "more each on the CPU"}


def config(args):
    return {"workload": "heisenberg_u1_chain_N100_maxdim1024_cutoff1e-12",
            "model": "S=1/2 Heisenberg OBC, MPO w=5, U(1) Sz=0, Neel start",
            "sites": N_SITES, "maxdim": MAXDIM, "ramp": RAMP, "cutoff": CUTOFF,
            "krylovdim": KRYLOVDIM, "maxiter": MAXITER, "precision": args.precision,
            "parallelism": f"replicas{args.gpus}",
            "l2": "working set (environments of all 100 sites, ~0.3 GB) larger than L2"}


# ------------------------------------------------------------------------------------
# our arm
# ------------------------------------------------------------------------------------

def save_state(path, psi):
    import numpy as np
    t, lk = download_state(psi)
    np.savez(path, *(t + lk))


def load_state(tn, ctx, path, pq):
    import numpy as np
    z = np.load(path)
    arrs = [z[f"arr_{i}"] for i in range(2 * N_SITES + 1)]
    return tn.MPS(arrs[:N_SITES], arrs[N_SITES:], pq, 0, ctx)


def run_partial(tn, ctx, env, args):
    """Profiling aid: the first K left-to-right bond updates of the timed sweep."""
    for p in range(args.partial_updates):
        tn.update_position_(env, tn.eig_solver, p, 2, "left", maxdim=MAXDIM, cutoff=CUTOFF,
                            solver_krylovdim=KRYLOVDIM, solver_maxiter=MAXITER)
    print(json.dumps({"partial_updates": args.partial_updates,
                      "launches": ctx.lib.tn_kernel_launches()}), flush=True)


def run_ours(args, world, rank, local, pg):
    import __graft_entry__ as g
    g.build()
    tn = g.load_package()
    if args.ttn_only:
        if rank == 0:
            print(json.dumps({"ttn": run_ttn(tn, local, args, world)}), flush=True)
        return
    if args.j1j2_chi2048:
        if rank == 0:
            print(json.dumps({"j1j2_chi2048": run_j1j2(tn, local, args)}), flush=True)
        return
    if args.svd_bond:
        if rank == 0:
            print(json.dumps({"svd_bond": run_svd_bond(tn, local, args)}), flush=True)
        return
    if args.quench_only:
        if rank == 0:
            print(json.dumps({"quench": run_quench(tn, local, args)}), flush=True)
        return
    ctx = tn.Context(local)
    if args.precision == "split":
        ctx.set_precision("split", args.slices)
    H, pq = heisenberg(tn, ctx)
    sw = tn.SweepData()
    if args.load_state:
        env = tn.StateEnvs(load_state(tn, ctx, args.load_state, pq), H)
        if args.partial_updates:
            run_partial(tn, ctx, env, args)
            return
    else:
        psi0 = tn.MPS.product(tn.models.neel_states(N_SITES), pq, ctx)
        env = tn.StateEnvs(psi0, H)
        for md in RAMP:  # prepare the converged state (not timed)
            tn.fullsweep_(env, tn.eig_solver, 2, sw, **sweep_kwargs(md))
    for _ in range(args.warmup):
        tn.fullsweep_(env, tn.eig_solver, 2, sw, **sweep_kwargs(MAXDIM))
    if args.save_state:
        save_state(args.save_state, env.getpsi())
        print(json.dumps({"saved": args.save_state, "maxlinkdim": sw.maxchi[-1]}), flush=True)
        return
    n0 = len(sw.stats)
    # kernels launched before the timed region (lets a profiler skip the preparation)
    print(f"launches_before_timed={ctx.lib.tn_kernel_launches()}", file=sys.stderr, flush=True)
    barrier(pg)
    t0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            tn.fullsweep_(env, tn.eig_solver, 2, sw, **sweep_kwargs(MAXDIM))
    wall = time.perf_counter() - t0
    barrier(pg)
    st = sw.stats[n0:]
    dev_s = sum(s["sweep_ms"] for s in st) / 1e3 / args.steps
    dev_s = allmax(pg, dev_s)
    heff_ms = sum(s["heff_ms"] for s in st)
    heff_fl = sum(s["heff_flops"] for s in st)
    gemm_ms = sum(s["gemm_ms"] for s in st)
    gemm_fl = sum(s["gemm_flops"] for s in st)
    gemm_n = sum(s["gemm_launches"] for s in st)
    launches = sum(s["kernel_launches"] for s in st)
    energy = sw.energy[-1]
    chi = sw.maxchi[-1]

    # end to end through the C ABI with host buffers: upload the MPS (charge blocks, as an
    # ITensors QN MPS holds them), build the environments, sweep, download the MPS blocks
    psi_t = env.getpsi()
    tensors, links = download_state(psi_t)
    blocks, _ = download_blocks(psi_t)
    del psi_t
    h2d = sum(b.size * 8 for b in blocks)
    e2e_times = []
    for _ in range(max(1, min(args.steps, 2))):
        t1 = time.perf_counter()
        p2 = tn.MPS.from_blocks(blocks, links, pq, 0, ctx)
        e2 = tn.StateEnvs(p2, H)
        s2 = tn.SweepData()
        tn.fullsweep_(e2, tn.eig_solver, 2, s2, **sweep_kwargs(MAXDIM))
        e2e_energy, e2e_chi = s2.energy[-1], s2.maxchi[-1]
        out = download_blocks(e2.getpsi())
        e2e_times.append(time.perf_counter() - t1)
        d2h = sum(b.size * 8 for b in out[0])
        del e2, p2
    e2e = allmax(pg, statistics.mean(e2e_times))

    if rank != 0:
        return
    pk = peaks()
    gemm_tflops = gemm_fl / max(gemm_ms, 1e-9) / 1e9
    if args.precision == "split":
        roof = {"bound": "tensor", "achieved": gemm_tflops, "peak": pk["bf16_tflops"],
                "unit": "TFLOP/s", "frac": gemm_tflops / pk["bf16_tflops"],
                "peak_note": "of measured bf16 (algorithmic FP64-equivalent flops, slice "
                             "products not counted)"}
    else:
        roof = {"bound": "fp64", "achieved": gemm_tflops, "peak": FP64_PEAK_NOMINAL_TFLOPS,
                "unit": "TFLOP/s", "frac": gemm_tflops / FP64_PEAK_NOMINAL_TFLOPS,
                "peak_note": "of nominal GB300 FP64 (no measured FP64 peak on this pool)"}
    roof["kernel"] = ("tcgen05 split-precision grouped GEMM of H_eff (two launches per matvec)"
                      if args.precision == "split" else
                      "FP64 grouped block-sparse GEMM of H_eff (two launches per matvec)")
    roof["flops_per_launch"] = gemm_fl / max(gemm_n, 1)
    roof["ms_per_launch"] = gemm_ms / max(gemm_n, 1)
    # DRAM bytes (read + write) per launch of this kernel at this workload: the mean over
    # 20 consecutive launches of one ncu capture (dram__bytes_read.sum +
    # dram__bytes_write.sum, profiles/split_gemm_traffic_heisenberg_N100.md); per launch
    # like `achieved`
    roof["traffic"] = 2.808704e6 if args.precision == "split" else None
    roof["traffic_unit"] = "bytes per launch (mean of 20 launches, one ncu capture)"
    share = {k: sum(s[k] for s in st) / max(sum(s["sweep_ms"] for s in st), 1e-9)
             for k in ("heff_ms", "svd_ms", "env_ms", "lanczos_ms", "pack_ms", "gemm_ms")}
    dominant = max(("svd_ms", "heff_ms", "lanczos_ms", "env_ms"), key=lambda k: share[k])
    dom = {"svd_ms": {"kernel": "block SVD per bond: svd_qrj_kernel (one CTA per charge block: "
                                "double-float QR with pivoting, FP32 Jacobi presolve, double-float "
                                "polish) or the multi-SM pipeline (blocked QR + cooperative "
                                "block-pair Jacobi), split tuned per block-size histogram",
                      "bound": "FP32 pipe of one SM per charge block (latency-bound at chi~180: "
                               "7-9 blocks of <= ~110 columns per bond)"},
           "heff_ms": {"kernel": "split_pack_kernel + split_gemm_kernel + combine_kernel",
                       "bound": "tensor (see roofline)"},
           "lanczos_ms": {"kernel": "gs_pass_kernel", "bound": "hbm"},
           "env_ms": {"kernel": "environment GEMMs", "bound": "tensor"}}[dominant]
    dom["share"] = share[dominant]
    # the block SVD against the FP32 pipe (every SVD phase runs there: FP32 Jacobi presolve,
    # double-float QR, polish and Q V; the multi-SM path's GEMMs on the tensor cores)
    svd_fl = sum(s.get("svd_small_flops", 0.0) + s.get("svd_gemm_flops", 0.0) +
                 s.get("svd_jacobi_flops", 0.0) for s in st)
    svd_ms = sum(s["svd_ms"] for s in st)
    svd_roof = {"bound": "fp32", "achieved": svd_fl / max(svd_ms, 1e-9) / 1e9,
                "peak": FP32_PEAK_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                "frac": svd_fl / max(svd_ms, 1e-9) / 1e9 / FP32_PEAK_NOMINAL_TFLOPS,
                "peak_note": "of nominal FP32 (152 SMs x 128 lanes x 2 x 2.07 GHz; no measured "
                             "FP32 peak on this pool)",
                "flops_per_sweep": svd_fl / args.steps,
                "flops_note": "algorithmic FP64-equivalent flops of the block SVDs (QR, Jacobi "
                              "sweeps as run, Gram-Schmidt, R^T V, Q V; a double-float operation "
                              "counts once) over the CUDA-event time of the SVD"}
    if dominant == "svd_ms":
        dom["achieved_tflops"] = svd_roof["achieved"]
        dom["frac_of_nominal_fp32"] = svd_roof["frac"]
    res = {
        "metric": METRIC, "value": dev_s, "unit": "s/sweep", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64 (bf16-slice tensor-core GEMMs)",
        "data": "synthetic", "config": config(args),
        "heff_tflops": heff_fl / max(heff_ms, 1e-9) / 1e9,
        "heff_ms_per_sweep": heff_ms / args.steps,
        "time_share": share,
        "matvecs_per_sweep": sum(s["matvecs"] for s in st) / args.steps,
        "krylov_hbm_gbs": sum(s["krylov_bytes"] for s in st)
                          / max(sum(s["lanczos_ms"] for s in st), 1e-9) / 1e6,
        "krylov_hbm_note": "algorithmic bytes of the Lanczos vector kernels (each element read "
                           "or written once per launch) over their CUDA-event time",
        "energy": energy, "maxlinkdim": chi, "wall_s_per_sweep": wall / args.steps,
        "gpu_launches": launches,
        "roofline": roof,
        "svd_roofline": svd_roof,
        "dominant_kernel": dom,
        "clocks": clk.summary(),
        "e2e": {"value": e2e, "unit": "s/sweep", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "what": "upload the MPS charge blocks from host + build environments + one sweep "
                        "+ download the MPS charge blocks"},
    }
    res["svd_schedule"] = ctx.svd_schedule()
    if args.precision == "split" and not args.no_fp64_compare:
        res["fp64_compare"] = fp64_compare(tn, ctx, H, pq, tensors, links, local)
    if world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline_from(tensors, links)
        res["cpu_baseline"] = cb
        # the same sweep from the same state on the GPU (the e2e leg) and on the CPU oracle
        res["vs_cpu"] = {"dE_rel_vs_cpu": abs(e2e_energy - cb["energy"]) / abs(cb["energy"]),
                         "same_bond_dims_vs_cpu": int(e2e_chi) == int(cb["maxlinkdim"]),
                         "gpu_energy": e2e_energy, "cpu_energy": cb["energy"],
                         "gpu_maxlinkdim": int(e2e_chi), "cpu_maxlinkdim": cb["maxlinkdim"]}
    if not args.no_ttn:
        res["ttn"] = run_ttn(tn, local, args, world)
    if not args.no_quench:
        try:
            res["quench"] = run_quench(tn, local, args)
        except Exception as e:  # an extra leg: report it, keep the headline line
            res["quench"] = {"error": f"{type(e).__name__}: {e}"}
    if not args.no_j1j2:
        try:
            res["j1j2_chi2048"] = run_j1j2(tn, local, args)
        except Exception as e:  # an extra leg: report it, keep the headline line
            res["j1j2_chi2048"] = {"error": f"{type(e).__name__}: {e}"}
    print(json.dumps(res), flush=True)


# J1-J2 cylinder at chi = 2048: the 6 x 16 cylinder (Ly = 6 periodic, Lx = 16 open, 96 sites,
# MPO bond dimension 26 in the bulk), J2/J1 = 0.5, U(1), cutoff 1e-10
J1J2_LX, J1J2_LY = 16, 6
J1J2_CHI = 2048
# two-site DMRG from a Neel product state grows the bond dimension about fourfold per sweep
# (4, 16, 64, 256, 1024, 2048): six ramp sweeps reach chi = 2048 in the bulk
J1J2_RAMP = [256, 512, 1024, 2048, 2048, 2048]


def run_j1j2(tn, local, args):
    """Ramp to chi = 2048 (untimed), then one sweep from the same state on the split path and
    on the FP64 GPU path: sweep time, H_eff time and TFLOP/s, SVD time and flops, energies,
    truncation errors and the state overlap.  States stay on the device (one context whose
    precision is switched between the two sweeps)."""
    Lx = args.j1j2_lx
    N = Lx * J1J2_LY
    terms = tn.models.j1j2_cylinder_terms(Lx, J1J2_LY)
    W, delta, pq = tn.models.mpo_from_terms(N, terms)
    neel = [((i // J1J2_LY) + (i % J1J2_LY)) % 2 for i in range(N)]
    ctx = tn.Context(local, precision="split", slices=args.slices)
    H = tn.MPO(W, delta, pq, ctx)
    env = tn.StateEnvs(tn.MPS.product(neel, pq, ctx), H)
    sw = tn.SweepData()
    t0 = time.perf_counter()
    for md in J1J2_RAMP:
        tn.fullsweep_(env, tn.eig_solver, 2, sw, maxdim=md, cutoff=1e-10, outputlevel=0)
    prep = time.perf_counter() - t0
    psi = env.getpsi()
    del env
    out = {"workload": f"j1j2_cylinder_{J1J2_LY}x{Lx}_J2_0.5_u1_chi{J1J2_CHI}_cutoff1e-10",
           "sites": N, "mpo_bond_dim": int(max(w.shape[0] for w in W)), "ramp": J1J2_RAMP,
           "prepare_s": prep, "chi_start": int(psi.maxlinkdim()),
           "note": "one sweep from the same ramped state on each path (2 (N - 1) bond updates)"}
    final = {}
    for prec in ("split", "fp64"):
        ctx.set_precision(prec, args.slices)
        e = tn.StateEnvs(psi, H)
        s = tn.SweepData()
        tn.fullsweep_(e, tn.eig_solver, 2, s, maxdim=J1J2_CHI, cutoff=1e-10, outputlevel=0)
        st = s.stats[-1]
        out[prec] = {"sweep_s": st["sweep_ms"] / 1e3, "heff_s": st["heff_ms"] / 1e3,
                     "heff_tflops": st["heff_flops"] / max(st["heff_ms"], 1e-9) / 1e9,
                     "gemm_s": st["gemm_ms"] / 1e3, "pack_s": st["pack_ms"] / 1e3,
                     "gemm_tflops": st["gemm_flops"] / max(st["gemm_ms"], 1e-9) / 1e9,
                     "svd_s": st["svd_ms"] / 1e3, "env_s": st["env_ms"] / 1e3,
                     "lanczos_s": st["lanczos_ms"] / 1e3,
                     "svd_gemm_flops": st.get("svd_gemm_flops", 0.0),
                     "svd_jacobi_flops": st.get("svd_jacobi_flops", 0.0),
                     "svd_sweeps_max": [st.get("svd_sweeps32", 0), st.get("svd_sweeps_df", 0)],
                     # algorithmic SVD flops (GEMMs + Jacobi rotations, FP64-equivalent) over
                     # the whole SVD time (QR panels and small-block kernels included)
                     "svd_algorithmic_tflops": (st.get("svd_gemm_flops", 0.0) +
                                                st.get("svd_jacobi_flops", 0.0) +
                                                st.get("svd_small_flops", 0.0))
                                               / max(st["svd_ms"], 1e-9) / 1e9,
                     "energy": s.energy[-1], "maxlinkdim": s.maxchi[-1],
                     "maxtruncerr": s.maxtruncerr[-1]}
        final[prec] = e.getpsi()
        del e
    out["svd_schedule"] = ctx.svd_schedule()
    ps, pd = final["split"], final["fp64"]
    out["overlap_split_fp64"] = abs(ps.inner(pd)) / math.sqrt(ps.inner(ps) * pd.inner(pd))
    out["dE_rel"] = abs(out["split"]["energy"] - out["fp64"]["energy"]) / abs(out["fp64"]["energy"])
    out["speedup_sweep_split_vs_fp64"] = out["fp64"]["sweep_s"] / out["split"]["sweep_s"]
    out["speedup_heff_split_vs_fp64"] = out["fp64"]["heff_s"] / out["split"]["heff_s"]
    out["same_bond_dims"] = (out["split"]["maxlinkdim"] == out["fp64"]["maxlinkdim"] and
                             ps.linkdims() == pd.linkdims())
    ctx.set_precision("split", args.slices)
    return out


# Real-time two-site TDVP quench (ComplexF64): the N = 64 Heisenberg chain from the Neel
# state, tau = -0.05i, maxdim 512, cutoff 1e-9, Krylov dimension 30.  The state is first
# evolved (untimed) to t = 5 in steps of 0.25, where the bond dimension has grown to ~100;
# then --steps sweeps of the workload's step are timed.
QUENCH_N, QUENCH_DT, QUENCH_CHI, QUENCH_CUTOFF, QUENCH_KRYLOV = 64, 0.05, 512, 1e-9, 30
QUENCH_PREP_DT, QUENCH_PREP_SWEEPS = 0.25, 20
QUENCH_CPU_BONDS = 6


def run_quench(tn, local, args):
    """Complex TDVP sweeps on the GPU from one prepared state, in split precision (complex
    H_eff products through the bf16-slice tensor-core GEMM, unsigned complex form) and in
    FP64 (DFMA), and the oracle's complex restatement timed on a bounded sample of the same
    sweep.  Environment updates, the realified block SVD and the Krylov exponential are FP64
    on both paths."""
    import numpy as np
    N = QUENCH_N
    ctx = tn.Context(local, precision="split", slices=args.slices)
    W, delta, pq = tn.models.mpo_from_terms(N, tn.models.heisenberg_chain_terms(N))
    H = tn.MPO(W, delta, pq, ctx)
    eng = tn.TDVPEngine(tn.MPS.product(tn.models.neel_states(N), pq, ctx), H)
    kw = dict(maxdim=QUENCH_CHI, cutoff=QUENCH_CUTOFF, solver_krylovdim=QUENCH_KRYLOV)
    t0 = time.perf_counter()
    for _ in range(QUENCH_PREP_SWEEPS):
        tn.tdvpsweep_(eng, -1j * QUENCH_PREP_DT, **kw)
    prep = time.perf_counter() - t0
    psi0 = eng.getpsi()
    del eng
    e_neel = -0.25 * (N - 1)  # <Neel| sum S_i . S_i+1 |Neel>, conserved by the evolution
    out = {"workload": f"heisenberg_chain_N{N}_neel_quench_tau-{QUENCH_DT}i_maxdim{QUENCH_CHI}"
                       f"_cutoff{QUENCH_CUTOFF:g}_krylov{QUENCH_KRYLOV}",
           "dtype": "c128 (planar complex FP64)",
           "prepare": f"{QUENCH_PREP_SWEEPS} untimed sweeps of tau = -{QUENCH_PREP_DT}i (t = "
                      f"{QUENCH_PREP_SWEEPS * QUENCH_PREP_DT:g})",
           "prepare_s": prep, "chi_start": int(psi0.maxlinkdim())}
    final = {}
    for prec in ("split", "fp64"):
        ctx.set_precision(prec, args.slices)
        e = tn.TDVPEngine(psi0, H)
        sweeps = []
        # kernel launches of this library before the path's first timed sweep (the offset of
        # an ncu launch-list capture of that sweep)
        out[f"launches_before_{prec}"] = int(ctx.lib.tn_kernel_launches())
        for _ in range(max(args.steps, 1)):
            tn.tdvpsweep_(e, -1j * QUENCH_DT, **kw)
            st = e.swdata.stats[-1]
            sweeps.append({"sweep_s": st["sweep_ms"] / 1e3, "heff_s": st["heff_ms"] / 1e3,
                           "gemm_s": st["gemm_ms"] / 1e3, "svd_s": st["svd_ms"] / 1e3,
                           "env_s": st["env_ms"] / 1e3, "krylov_s": st["lanczos_ms"] / 1e3,
                           "matvecs": st["matvecs"], "kernel_launches": st["kernel_launches"],
                           "heff_tflops": st["heff_flops"] / max(st["heff_ms"], 1e-9) / 1e9,
                           "maxlinkdim": e.maxchi(), "energy": e.getenergy(),
                           "maxtruncerr": e.sweeperror()})
            if len(sweeps) == 1:
                first_sz = [float(v) for v in tn.measure(e.getpsi(), "Sz")]
        psi = e.getpsi()
        final[prec] = psi
        out[prec] = {"timed_sweeps": sweeps, "first_sz": first_sz,
                     "sweep_s_mean": sum(x["sweep_s"] for x in sweeps) / len(sweeps),
                     "heff_s_mean": sum(x["heff_s"] for x in sweeps) / len(sweeps),
                     "energy_drift_rel": abs(sweeps[-1]["energy"] - e_neel) / abs(e_neel),
                     "sz": [float(v) for v in tn.measure(psi, "Sz")],
                     "norm": abs(psi.inner(psi))}
        del e
    ctx.set_precision("split", args.slices)
    ps, pd = final["split"], final["fp64"]
    out["max_sz_diff_split_fp64"] = float(np.abs(np.array(out["split"]["sz"]) -
                                                 np.array(out["fp64"]["sz"])).max())
    out["total_sz"] = float(sum(out["split"]["sz"]))
    out["overlap_split_fp64"] = abs(ps.inner(pd))
    out["same_bond_dims"] = ps.linkdims() == pd.linkdims()
    out["speedup_sweep_split_vs_fp64"] = out["fp64"]["sweep_s_mean"] / out["split"]["sweep_s_mean"]
    out["speedup_heff_split_vs_fp64"] = out["fp64"]["heff_s_mean"] / out["split"]["heff_s_mean"]
    if not args.no_cpu_baseline:
        cb = quench_cpu_sample(psi0)
        # the GPU's first sweep from psi0 (split path) against the oracle's sweep from psi0
        sp = out["split"]
        out["vs_cpu"] = {"max_sz_diff": float(np.abs(np.array(sp["first_sz"]) -
                                                     np.array(cb.pop("sz"))).max()),
                         "dE_rel": abs(sp["timed_sweeps"][0]["energy"] - cb["energy"]) /
                                   abs(cb["energy"]),
                         "same_bond_dims": sp["timed_sweeps"][0]["maxlinkdim"] == cb["maxlinkdim"]}
        out["cpu_baseline"] = cb
        out["speedup_vs_cpu_port"] = cb["value"] / out["split"]["sweep_s_mean"]
    for prec in ("split", "fp64"):
        del out[prec]["sz"]
        del out[prec]["first_sz"]
    return out


def quench_cpu_sample(psi):
    """One full complex TDVP sweep of the oracle (numpy FP64) from the same state on the host
    cores (right environments built untimed): its time, and its <S^z_i>, energy and bond
    dimension for the comparison with the GPU's first sweep from that state."""
    import numpy as np
    from oracle import tn_oracle as O
    N = psi.N
    tensors, links = download_state(psi)
    st = O.MPS([np.asarray(t) for t in tensors], [np.asarray(q, dtype=np.int64) for q in links],
               O.SPIN_HALF_Q.copy(), center=0)
    env = O.StateEnvs(st, O.heisenberg_mpo(N))
    env.position(0, 2)
    sw = O.SweepData()
    t0 = time.perf_counter()
    O.tdvp_sweep(env, sw, -1j * QUENCH_DT, QUENCH_CHI, QUENCH_CUTOFF, 1, QUENCH_KRYLOV, 100, 1e-12)
    dt = time.perf_counter() - t0
    return {"value": dt, "unit": "s/sweep", "cores": cores(), "kind": "port", "dense": True,
            "energy": sw.energy[-1], "maxlinkdim": int(env.psi.maxlinkdim()),
            "sz": [float(v) for v in O.expect_local(env.psi, np.diag([0.5, -0.5]))],
            "sample": f"one full complex two-site TDVP sweep ({2 * (N - 1)} bond updates) of the "
                      "numpy FP64 oracle (dense tensors with charge labels; OpenBLAS threads = "
                      "all host cores) from the same state"}


# one bond's charge blocks at chi ~ 2048 (the sizes of the largest bond of the 6 x 16 J1-J2
# cylinder): rows x cols of the seven largest blocks
SVD_BOND_SHAPES = [(1200, 1100), (1150, 1050), (1100, 1000), (900, 850), (600, 450), (300, 250),
                   (150, 126)]


def run_svd_bond(tn, local, args):
    """The block SVD of one chi ~ 2048 bond (seeded synthetic blocks graded over 8 decades on
    both sides, as a two-site tensor between Schmidt bases) through tn_svd_truncate, in the
    context's precision: wall time per call and the SVD's work counters."""
    import numpy as np
    rng = np.random.default_rng(7)
    blocks = []
    for r, c in SVD_BOND_SHAPES:
        dl = 10.0 ** (-8.0 * (np.arange(r) / r) ** 0.8) * rng.uniform(0.7, 1.3, r)
        dr = 10.0 ** (-8.0 * (np.arange(c) / c) ** 0.8) * rng.uniform(0.7, 1.3, c)
        blocks.append(dl[:, None] * rng.standard_normal((r, c)) * dr[None, :])
    ctx = tn.Context(local, precision=args.precision, slices=args.slices)
    walls = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        kept, _, err = tn.svd_truncate(blocks, cutoff=1e-12, ctx=ctx)
        walls.append(time.perf_counter() - t0)
    return {"workload": "block SVD of one chi~2048 bond (7 charge blocks, largest 1200 x 1100)",
            "precision": args.precision, "calls": len(walls), "wall_s": walls,
            "kept": [int(k) for k in kept], "truncerr": float(err)}


def fp64_compare(tn, ctx, H, pq, tensors, links, local):
    """One sweep from the same state on the split path and on the FP64 GPU path."""
    out = {}
    ctx64 = tn.Context(local, precision="fp64")
    H64, _ = heisenberg(tn, ctx64)
    final = {}
    for name, c, h in (("split", ctx, H), ("fp64", ctx64, H64)):
        e = tn.StateEnvs(tn.MPS(tensors, links, pq, 0, c), h)
        sw = tn.SweepData()
        tn.fullsweep_(e, tn.eig_solver, 2, sw, **sweep_kwargs(MAXDIM))
        st = sw.stats[-1]
        out[name] = {"sweep_s": st["sweep_ms"] / 1e3, "energy": sw.energy[-1],
                     "heff_ms": st["heff_ms"], "svd_ms": st["svd_ms"], "maxlinkdim": sw.maxchi[-1],
                     "maxtruncerr": sw.maxtruncerr[-1]}
        final[name] = download_state(e.getpsi())
        del e
    # state overlap |<psi_split|psi_fp64>| of the two (normalised) results, on the GPU
    ps = tn.MPS(final["split"][0], final["split"][1], pq, 0, ctx)
    pd = tn.MPS(final["fp64"][0], final["fp64"][1], pq, 0, ctx)
    out["overlap_split_fp64"] = abs(ps.inner(pd)) / math.sqrt(ps.inner(ps) * pd.inner(pd))
    del ps, pd
    out["speedup_split_vs_fp64"] = out["fp64"]["sweep_s"] / out["split"]["sweep_s"]
    out["heff_speedup_split_vs_fp64"] = out["fp64"]["heff_ms"] / max(out["split"]["heff_ms"], 1e-9)
    out["dE_rel"] = abs(out["split"]["energy"] - out["fp64"]["energy"]) / abs(out["fp64"]["energy"])
    out["same_bond_dims"] = out["split"]["maxlinkdim"] == out["fp64"]["maxlinkdim"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="split", choices=["fp64", "split"])
    ap.add_argument("--slices", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-ttn", action="store_true", help="skip the TTN (32-instance) leg")
    ap.add_argument("--ttn-only", action="store_true", help="run only the TTN leg")
    ap.add_argument("--ttn-instances", type=int, default=TTN_INSTANCES)
    ap.add_argument("--j1j2-chi2048", action="store_true",
                    help="only the J1-J2 cylinder comparison at chi = 2048 (split vs FP64)")
    ap.add_argument("--svd-bond", action="store_true",
                    help="only the block SVD of one chi ~ 2048 bond (--steps calls)")
    ap.add_argument("--no-quench", action="store_true",
                    help="skip the real-time TDVP quench (complex) leg of the default run")
    ap.add_argument("--quench-only", action="store_true",
                    help="only the real-time TDVP quench (complex) leg")
    ap.add_argument("--no-j1j2", action="store_true",
                    help="skip the chi = 2048 J1-J2 comparison leg of the default run")
    ap.add_argument("--j1j2-lx", type=int, default=J1J2_LX,
                    help="cylinder length of the J1-J2 leg (16: the 6 x 16 cylinder)")
    ap.add_argument("--save-state", default="", help="save the prepared MPS (npz) and exit")
    ap.add_argument("--load-state", default="", help="start from a saved MPS (no ramp)")
    ap.add_argument("--partial-updates", type=int, default=0,
                    help="with --load-state: only the first K bond updates (profiling)")
    args = ap.parse_args()
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    else:
        run_ours(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()

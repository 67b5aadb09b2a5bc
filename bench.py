"""Benchmark: SIMP iterations/s on the 2D plane-strain MBB half beam,
1024 x 512 Q4 (1,051,650 dofs), MMA update, filter radius 3, every solve to
an FP64 relative residual of 1e-8.

A step is one SIMP iteration (filter, moduli, solve, compliance and
sensitivities, filtered sensitivities, MMA update).  Steps are consecutive
iterations of one optimisation run, after W warm-up iterations.

  value : steps/s with the design resident in HBM (device time from CUDA
          events on the library's stream, summed over the step's phases)
  e2e   : steps/s through psf_simp_step_host with host buffers (design in,
          design + densities out, copies inside the timed region)

One process per GPU (replicas only: independent optimisation runs, no
collective on the data path).  `--impl reference` times the reference's CPU
algorithm (the oracle restatement built -O3 -fopenmp) on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "SIMP iters/s at 1M DOF, resid 1e-8: learned+mixed FCG vs plain FP64 GPU PCG"
UNIT = "SIMP iterations/s"
L2_BYTES = 129 * 1024 * 1024
KERNEL_NAME = {"ir_mg_f32": "mg_fcg_dw_kernel (persistent flexible CG on double-word (FP32-pair) vectors, "
                            "FP32 V(2,2) Chebyshev multigrid)",
               "csr_jacobi_f64": "pcg_csr_kernel (persistent FP64 Jacobi PCG on CSR)",
               "ebe_jacobi_f64": "pcg_ebe_kernel<double> (persistent matrix-free FP64 Jacobi PCG)",
               "ir_jacobi_f32": "pcg_ebe_kernel<float> (FP32 Jacobi inner iterations)"}


def workload(name="mbb2d", nx=None, ny=None, nz=None):
    """The problem and its description.  mbb2d: the 1M-dof MBB half beam (the
    headline); h8: the 3D H8 cantilever, 128x64x64 elements (1,635,075 dofs),
    OC, vf 0.15, filter radius 2."""
    from pansfem2_gb300 import problems as PB
    if name == "c1":
        nx, ny = nx or 60, ny or 30
        return PB.cantilever_q4(nx, ny), f"cantilever {nx}x{ny} Q4 plane strain, OC, R=1.5, vf=0.5, PCG 1e-10"
    if name == "h8":
        nx, ny, nz = nx or 128, ny or 64, nz or 64
        pr = PB.cantilever_h8(nx, ny, nz)
        desc = f"H8 cantilever {nx}x{ny}x{nz}, OC, R=2, vf=0.15"
        return pr, desc
    nx, ny = nx or 1024, ny or 512
    return PB.mbb_q4(nx, ny), f"MBB half beam {nx}x{ny} Q4 plane strain, MMA, R=3, vf=0.4"


def mg_levels(pr, coarse_dofs=40):
    """Node counts of the multigrid hierarchy (every axis coarsened to ceil(n/2)
    elements while all have at least 2, until a level has <= coarse_dofs dofs),
    as psf_mg.cu builds it."""
    from pansfem2_gb300 import problems as PB
    nd = PB.counts(pr)[2]
    dims = [pr["nx"], pr["ny"]] + ([pr["nz"]] if pr["kind"] == PB.H8_SOLID else [])
    nodes = lambda d: int(np.prod([x + 1 for x in d]))  # noqa: E731
    levels = [nodes(dims)]
    while True:
        if len(levels) > 1 and levels[-1] * nd <= coarse_dofs:
            break
        if any(x < 2 for x in dims):
            break
        dims = [(x + 1) // 2 for x in dims]
        levels.append(nodes(dims))
    return levels


def bytes_per_krylov_iteration(solver, pr, nnz, nfree):
    """Algorithmic HBM bytes of one Krylov iteration (every array a phase
    touches counted once per phase).
    Jacobi PCG (three phases): the operator, 12 B per stored entry, and 14
    vector passes (p = z + beta p: z, p read, p written; A p: p gathered, p
    read, Ap written; update: x, p, Ap, r, 1/D read, x, r, z written).
    Multigrid FCG (ir_mg_f32): Krylov phases on 8-byte double-word vectors,
    125 B/dof + 8 B/element (z and dot products: the cycle's result, q, r, p
    28; p and q = rs K x - beta q_prev: x, p, q read, p, q written 36 + E;
    update: x, p, r, q, D, fixed read, x, r, the next cycle's input and first
    sweep written 61), the fused level-0 V(2,2) work 34 B/dof + 8 B/element
    (each fused phase reads its level's vectors, diagonal, flags and moduli
    once), and per coarse level four stencil applications (9 blocks in 2D, 27
    in 3D, of nd x nd floats per node) plus 34 B/dof of level vectors."""
    from pansfem2_gb300 import problems as PB
    ne, nnodes, nd = PB.counts(pr)
    ndofs = nnodes * nd
    if solver == "csr_jacobi_f64":
        return 12 * nnz + 14 * 8 * nfree
    if solver == "ebe_jacobi_f64":
        return 8 * ne + 16 * ndofs + 11 * 8 * ndofs
    if solver == "ir_mg_f32":
        nb = 27 if pr["kind"] == PB.H8_SOLID else 9
        outer = 125 * ndofs + 8 * ne
        level0 = 34 * ndofs + 8 * ne
        coarse = sum(4 * nb * nd * nd * 4 * n + 34 * nd * n for n in mg_levels(pr)[1:-1])
        return outer + level0 + coarse
    # FP32 inner Jacobi iterations
    return 4 * ne + 8 * ndofs + 11 * 4 * ndofs


def max_over_ranks(values, world, device=None):
    """The elementwise maximum of this rank's timings over all ranks of the default process
    group (NCCL on the GPUs, gloo in the CPU tests); the values themselves for one rank.
    Every replica does the same work, so the slowest rank sets the job's time."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    if device is None:
        device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms.  __enter__ waits
    for the first sample so that the sampler is live before the work starts;
    window(t0, t1) (perf_counter times of the timed region) restricts the summary
    to the samples read during it (plus one sampling period)."""

    def __init__(self, index=0):
        self.index, self.rows, self.proc, self.win = index, [], None, None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            t_end = time.perf_counter() + 5.0
            while not self.rows and time.perf_counter() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def window(self, t0, t1):
        self.win = (t0, t1)

    def summary(self):
        rows = [r for _, r in self.rows]
        if self.win:
            t0, t1 = self.win
            inside = [r for t, r in self.rows if t0 <= t <= t1 + 0.25]
            before = [r for t, r in self.rows if t < t0]
            # a timed region shorter than the period: the sample read just before it
            rows = inside if inside else before[-1:]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows),
                "samples_total": len(self.rows)}


def run_device(pr, solver, warmup, steps, cg_eps, warm_start):
    import pansfem2_gb300 as P
    prob = P.Problem(pr)
    prob.setup_bc()
    prob.simp_begin(solver=solver, cg_eps=cg_eps, warm_start=warm_start)
    prob.warm_infos = [prob.simp_step() for _ in range(warmup)]
    prob.sync()
    infos = []
    l0 = P.kernel_launches()
    t0 = time.perf_counter()
    for _ in range(steps):
        infos.append(prob.simp_step())
    prob.sync()
    wall = time.perf_counter() - t0
    prob.t_region = (t0, t0 + wall)
    prob.launches = P.kernel_launches() - l0
    return prob, infos, wall


def run_e2e(pr, solver, warmup, steps, cg_eps, warm_start, sample_at=()):
    """The same SIMP iterations through the public host-buffer call: every step copies
    the design in from pinned host memory and the next design and densities out.
    Returns the designs entering the steps listed in sample_at."""
    import pansfem2_gb300 as P
    try:
        import torch
        pin = lambda n: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
    except Exception:
        pin = lambda n: np.empty(n)  # noqa: E731
    prob = P.Problem(pr)
    prob.setup_bc()
    prob.simp_begin(solver=solver, cg_eps=cg_eps, warm_start=warm_start)
    ne = prob.ne
    s_host, s_next, rho_host = pin(ne), pin(ne), pin(ne)
    s_host[:] = pr["vf"]
    for _ in range(warmup):
        prob.simp_step_host(s_host, s_next, rho_host)
        s_host[:] = s_next
    prob.sync()
    want = set(sample_at)
    designs = {}
    t0 = time.perf_counter()
    infos = []
    for k in range(steps):
        if k in want:
            designs[k] = s_host.copy()
        infos.append(prob.simp_step_host(s_host, s_next, rho_host))
        s_host[:] = s_next
    wall = time.perf_counter() - t0
    prob.close()
    return infos, wall, 8 * ne, 16 * ne, designs


def heaviside_beta_at(pr, it):
    """The projection sharpness iteration `it` of a SIMP run uses: psf_simp_step multiplies
    beta by beta_mult at the start of every iteration k with k % beta_every == 0, k = 0, 1, ..."""
    beta, every = float(pr.get("beta", 0.5)), int(pr.get("beta_every", 40))
    if every <= 0:
        return beta
    return beta * float(pr.get("beta_mult", 2.0)) ** (it // every + 1)


def fp64_at_designs(pr, solver, designs, cg_eps, first_iter=0, warm_start=False):
    """One SIMP iteration of the given solver from each given design: device seconds of the
    iteration (CUDA events of its phases), its compliance and its Krylov count.  Cold start
    (the plain FP64 PCG path's own mode): the iteration from the design itself.  Warm start:
    two iterations from the design, the second timed, its solve started from the first's
    displacement.  Design k entered iteration first_iter + k of the trajectory; with the
    Heaviside filter the fresh problem gets the projection sharpness beta of that iteration
    (the continuation multiplies beta at iterations 0, beta_every, 2 beta_every, ...), so both
    solvers see the same densities."""
    import pansfem2_gb300 as P
    out = {}
    for k, s0 in sorted(designs.items()):
        prk = dict(pr)
        if prk.get("heaviside"):
            prk["beta"] = heaviside_beta_at(pr, first_iter + k)
            prk["beta_every"] = 0
        with P.Problem(prk) as prob:
            prob.setup_bc()
            prob.simp_begin(solver=solver, cg_eps=cg_eps, warm_start=warm_start, s0=s0)
            info = prob.simp_step()
            if warm_start:
                info = prob.simp_step()
        out[k] = {"t": sum(info["phase_seconds"]), "f": info["f"], "iters": info["solve"]["iterations"]}
    return out


def oracle_first_iterations(pr, iters, eps, threads):
    """The reference's CPU algorithm (the oracle restatement built with the reference's stock
    flags, -O3 -fopenmp; its SpMV on `threads` OpenMP threads, the rest sequential as in
    CG.h) runs SIMP iterations 0 .. iters-1 of the problem in full: filter, numbering and
    assembly, ScalingCG to the relative residual eps, compliance and sensitivities, filtered
    sensitivities and the optimiser update.  Returns the per-iteration fields (densities,
    designs after the update, nodal displacements, compliance, CG counts) and the measured
    wall time of the whole run; nothing is scaled or extrapolated."""
    from oracle import build as ob
    from oracle import pyoracle as O
    ob.build()
    O.set_threads(threads, fast=True)
    full = dict(pr, cg_eps=eps, cg_itmax=100000)
    t0 = time.perf_counter()
    res = O.simp_run(full, iters, fields=True, fast=True)
    wall = time.perf_counter() - t0
    return res, wall


def gpu_first_iterations(pr, solver, iters, eps, warm_start):
    """SIMP iterations 0 .. iters-1 on the device from the uniform start (the iterations the
    oracle runs), with the fields read back after each one."""
    import pansfem2_gb300 as P
    out = {"f": [], "rho": [], "s": [], "u": [], "iters": [], "res": []}
    with P.Problem(pr) as prob:
        prob.setup_bc()
        prob.simp_begin(solver=solver, cg_eps=eps, warm_start=warm_start)
        for _ in range(iters):
            info = prob.simp_step()
            fl = prob.fields()
            out["f"].append(info["f"])
            out["iters"].append(info["solve"]["iterations"])
            out["res"].append(info["solve"]["rel_residual"])
            for k in ("rho", "s", "u"):
                out[k].append(fl[k])
    return out


def parity_report(gpu, orc, iters):
    """Per-iteration differences of the device run from the oracle's: densities (the filtered
    densities the solve used) and designs after the update as max-abs, compliance and nodal
    displacements as relative errors (2-norm)."""
    rho = [float(np.max(np.abs(gpu["rho"][k] - orc["rho"][k]))) for k in range(iters)]
    s = [float(np.max(np.abs(gpu["s"][k] - orc["s_after"][k]))) for k in range(iters)]
    f = [float(abs(gpu["f"][k] - orc["f"][k]) / abs(orc["f"][k])) for k in range(iters)]
    u = [float(np.linalg.norm(gpu["u"][k] - orc["u"][k]) / np.linalg.norm(orc["u"][k])) for k in range(iters)]
    return {"iterations": iters, "rho_max_abs": rho, "design_max_abs": s, "compliance_rel": f,
            "displacement_rel": u, "gpu_krylov_iterations": [int(v) for v in gpu["iters"]],
            "gpu_true_residual": [float(v) for v in gpu["res"]],
            "oracle_cg_iterations": [int(v) for v in orc["cg_iters"]],
            "oracle_true_residual": [float(v) for v in orc["true_res"]],
            "within_1e-6": bool(max(rho + s) <= 1e-6 and max(f) <= 1e-6)}


def cpu_sample_text(pr_desc, iters, eps, cg_iters, threads, wall):
    return (f"SIMP iterations 0-{iters - 1} of the {pr_desc} in full on the host (filter, numbering, CSR "
            f"assembly, ScalingCG to the relative residual {eps:g}: {'/'.join(str(int(v)) for v in cg_iters)} "
            f"CG iterations, compliance, sensitivities, optimiser update), oracle restatement of the reference "
            f"built -O3 -fopenmp, SpMV on {threads} threads; measured wall time {wall:.1f} s, not scaled")


HEAT_BATCH_METRIC = "aggregate instance-SIMP-iterations/s, batched heat-sink instances, resid 1e-8"


def bench_heat_batch(args, rank, world):
    """256 independent heat-sink instances (sides uniform in {64,...,384}, seeded
    patch edges/positions, vf in [0.3, 0.5]), one SIMP iteration of all of them
    per CUDA-graph replay.  Compared with the same instances run one by one
    through the single-problem path with plain FP64 Jacobi PCG (CSR)."""
    from pansfem2_gb300 import problems as PB
    insts = PB.heat_batch(args.instances, seed=rank)
    ne = sum(d["side"] ** 2 for d in insts)
    nn = sum((d["side"] + 1) ** 2 for d in insts)
    config = {"workload": f"{len(insts)} heat-sink instances, sides in {{64,96,128,192,256,384}}, OC, R=1.5, "
                          f"kmin=1e-3, p=3", "instances": len(insts), "elements": ne, "dofs": nn,
              "residual": "FP64 relative 1e-8", "parallelism": f"replicas{world}",
              "l2": "working set ~1 GB, larger than L2"}
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import build as ob
        from oracle import pyoracle as O
        ob.build()
        thr = ncpus()
        O.set_threads(thr, fast=True)
        # bounded sample, timed whole: 2 instances of each size, one full SIMP iteration each
        # (ScalingCG to 1e-8); one step = the whole sample
        sample = []
        for side in (64, 96, 128, 192, 256, 384):
            sample += [d for d in insts if d["side"] == side][:2]
        t0 = time.perf_counter()
        for d in sample:
            pr = PB.heatsink_q4(d["side"], d["side"], patch_w=d["patch_w"], patch_i0=d["patch_i0"], edge=d["edge"],
                                vf=d["vf"], cg_eps=1e-8)
            O.simp_run(pr, 1, fast=True)
        wall = time.perf_counter() - t0
        v = len(sample) / wall
        print(json.dumps({"impl": "reference", "metric": HEAT_BATCH_METRIC, "value": v,
                          "unit": "instance-iterations/s", "n_gpus": args.gpus, "steps": 1,
                          "warmup": 0, "ms_per_step": 1e3 * wall, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                          "config": config, "requested": {"steps": args.steps, "warmup": args.warmup},
                          "cpu_baseline": {"value": v, "unit": "instance-iterations/s", "cores": thr, "kind": "port",
                                           "sample": f"SIMP iteration 0 of {len(sample)} instances (2 of each size, "
                                                     f"not the batch's size mix), ScalingCG to 1e-8, measured wall "
                                                     f"time {wall:.1f} s"},
                          "e2e": {"value": v, "unit": "instance-iterations/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import pansfem2_gb300 as P
    from pansfem2_gb300 import autotune
    from pansfem2_gb300.batch import HeatBatch
    P.load()
    (threads, cluster), tune_times = autotune.tune_batch(insts, iters=1, warmup=1)
    with ClockSampler(local) as clk:
        with HeatBatch(insts, threads=threads, cluster=cluster) as B:
            B.begin(cg_eps=1e-8)
            B.step(args.warmup)
            done = B.results()["done"]
            l0 = P.kernel_launches()
            t0 = time.perf_counter()
            # one replay per iteration; an instance counts for the iterations it entered
            # unconverged (a converged one keeps its design, as the samples leave their loop,
            # and every phase returns at once for it)
            sides = np.array([d["side"] for d in insts])
            dev_t, active, t_first, bytes_solve, last_active = 0.0, 0, None, 0.0, 0
            for step in range(args.steps):
                live = done == 0
                active += int(np.sum(live))
                if live.any():
                    last_active = step + 1
                t = B.step(1)
                t_first = t if t_first is None else t_first   # the first timed iteration alone
                dev_t += t
                r_step = B.results()
                done = r_step["done"]
                # algorithmic bytes of this iteration's solves: per node and FCG iteration ~250 B
                # (double-word Krylov vectors 112 B, FP32 level-0 V(2,2) 100 B, coarse levels ~1/3
                # of level 0), over the instances that ran it
                bytes_solve += float(np.sum(np.where(live, r_step["iters"], 0) * (sides + 1.0) ** 2 * 250.0))
            clk.window(t0, time.perf_counter())
            nlaunch = P.kernel_launches() - l0
            res = B.results()
    # e2e: the same iterations (a fresh batch from the same initial designs, the same warm-up)
    # through the public API, each step followed by the read-back of its results
    with HeatBatch(insts, threads=threads, cluster=cluster) as B:
        B.begin(cg_eps=1e-8)
        B.step(args.warmup)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            B.step(1)
            r = B.results()
        e2e_t = time.perf_counter() - t0
    dev_t, e2e_t = max_over_ranks([dev_t, e2e_t], world)
    n = len(insts)
    value = world * active / dev_t
    its = res["iters"]
    peak, peak_kind = peaks()
    out = {"metric": HEAT_BATCH_METRIC, "value": value, "unit": "instance-iterations/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_t / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 cycle / f64 FCG",
           "data": "synthetic (seeded instances)",
           "config": dict(config, threads_per_cta=threads, ctas_per_instance=cluster),
           "clocks": clk.summary(), "gpu_launches": int(nlaunch),   # the graph's kernel nodes per replay
           "autotune": {"batch_threads_x_cluster": tune_times},
           "detail": {"active_instance_iterations": active, "converged_at_end": int(np.sum(res["done"] != 0)),
                      "iterations_until_all_converged": last_active,
                      "solve_iterations_mean": float(np.mean(its)), "solve_iterations_max": int(np.max(its)),
                      "true_residual_max": float(np.max(res["res"])), "all_converged": bool((res["conv"] == 1).all())},
           "roofline": {"bound": "hbm", "achieved": None, "peak": peak, "unit": "GB/s", "frac": None,
                        "traffic": None, "kernel": "solve_batch (one CTA per instance)",
                        "bytes_solves": bytes_solve, "peak_source": peak_kind,
                        "note": "achieved = algorithmic bytes of every timed solve / the timed device time of "
                                "all phases, a lower bound on the solve kernel's own rate"},
           "e2e": {"value": world * active / e2e_t, "unit": "instance-iterations/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 8 * 8 * n}}
    out["roofline"]["achieved"] = bytes_solve / dev_t / 1e9
    out["roofline"]["frac"] = out["roofline"]["achieved"] / peak
    if not args.no_compare and rank == 0:
        # the same instances one by one, plain FP64 Jacobi PCG through the single-problem path, timed
        # at the first timed iteration (after the same warm-up); the batch's own time for that one
        # iteration is the like-for-like comparison (later iterations of converging designs are cheaper)
        t_tot, n_done = 0.0, 0
        for d in insts:
            pr = PB.heatsink_q4(d["side"], d["side"], patch_w=d["patch_w"], patch_i0=d["patch_i0"], edge=d["edge"],
                                vf=d["vf"])
            prob, infos, wall = run_device(pr, "csr_jacobi_f64", args.warmup, 1, 1e-8, False)
            prob.close()
            t_tot += sum(infos[0]["phase_seconds"])
            n_done += 1
        first_rate = world * n / t_first
        out["one_by_one_fp64_pcg"] = {"value": n_done / t_tot, "unit": "instance-iterations/s",
                                      "solver": "csr_jacobi_f64",
                                      "batched_first_timed_iteration": first_rate,
                                      "speedup_first_timed_iteration": first_rate / (n_done / t_tot),
                                      "note": f"device time of SIMP iteration {args.warmup} of each instance (after "
                                              f"{args.warmup} warm-up iterations) against the batch's time for the same "
                                              "iteration"}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def learned_metric(nx, ny):
    dofs = 2 * (nx + 1) * (ny + 1)
    size = f"{dofs / 1e6:.2f}M" if dofs >= 1e6 else f"{dofs / 1e3:.0f}K"
    return f"SIMP iters/s at {size} DOF ({nx}x{ny} MBB), resid 1e-8: learned FCG vs Jacobi PCG"


def harvest_and_train(nx, ny, pairs, train_steps, seed=0):
    """Training pairs harvested from the method's own multigrid FCG solves along seeded SIMP runs
    of the nx x ny MBB beam (volume fraction uniform in [0.3, 0.6], point loads on the right
    edge, designs of the first iterations), then the U-Net trained on the GPU (scale-free energy
    loss, Adam).  Returns (network, harvest seconds, training seconds, loss history)."""
    import pansfem2_gb300 as P
    from pansfem2_gb300 import learned as Ln
    from pansfem2_gb300 import problems as PB
    H, W = nx + 1, ny + 1
    rng = np.random.default_rng(seed)
    ts = Ln.TrainSet(H, W, pairs)
    t0 = time.perf_counter()
    runs, iters_per_run = 8, 24
    per_design = max(1, pairs // (runs * (iters_per_run // 2)))
    while len(ts) < pairs:
        pr = PB.mbb_q4(nx, ny, vf=float(rng.uniform(0.3, 0.6)), load_right=int(rng.integers(ny // 4, ny + 1)))
        with P.Problem(pr) as prob:
            prob.setup_bc()
            prob.attach_learned(None, pre_mg=True, nu_post=1, use_net=False)
            prob.simp_begin(solver="ir_mg_f32", cg_eps=1e-8, warm_start=True)
            for k in range(iters_per_run):
                prob.simp_step()
                if k % 2 == 1 and len(ts) < pairs:
                    prob.harvest(ts, min(per_design, pairs - len(ts)), iters=[0, 1, 2, 3, 4, 6, 8, 12, 16])
    t_harvest = time.perf_counter() - t0
    net = Ln.UNet(H, W, batch=8, seed=3)
    t0 = time.perf_counter()
    hist = Ln.train(net, ts, train_steps, batch=8, lr=1e-3, seed=5, loss="angle")
    t_train = time.perf_counter() - t0
    ts.close()
    return net, t_harvest, t_train, hist


def learned_leg(pr, nx, ny, warmup, steps, eps, fp64_value, fp64_iters, mg_value, pairs=400, train_steps=1500):
    """The learned preconditioner on the headline problem: the U-Net is trained on a 512 x 256
    beam (harvest + training on the GPU, timed and reported), and, being fully convolutional,
    its parameters run on this grid; the learned flexible CG then runs the same SIMP window as
    the headline (W warm-up iterations, K timed), with the Jacobi PCG fallback after twice the
    plain FP64 PCG's iteration count on a stall."""
    import pansfem2_gb300 as P
    from pansfem2_gb300 import learned as Ln
    tnx, tny = 512, 256
    net_t, t_h, t_t, hist = harvest_and_train(tnx, tny, pairs, train_steps)
    net = Ln.UNet(nx + 1, ny + 1, batch=1, seed=3)
    net.set_params(net_t.get_params())
    net.out_scale = net_t.out_scale
    net_t.close()
    limit = int(2 * fp64_iters) if fp64_iters else 0
    with P.Problem(pr) as prob:
        prob.setup_bc()
        prob.attach_learned(net, pre_mg=True, nu_post=1, fallback_after=limit)
        prob.simp_begin(solver="ir_learned_f32", cg_eps=eps, warm_start=True)
        for _ in range(warmup):
            prob.simp_step()
        prob.sync()
        l0 = P.kernel_launches()
        infos = [prob.simp_step() for _ in range(steps)]
        nl = P.kernel_launches() - l0
    net.close()
    t = sum(sum(i["phase_seconds"]) for i in infos)
    v = steps / t
    return {"solver": "ir_learned_f32", "value": v, "unit": UNIT,
            "krylov_iterations": int(sum(i["solve"]["iterations"] for i in infos)),
            "fell_back": int(sum(i["solve"]["fell_back"] for i in infos)),
            "fallback_after": limit, "true_residual_max": max(i["solve"]["rel_residual"] for i in infos),
            "f_last": infos[-1]["f"], "kernel_launches": int(nl),
            "training": {"grid": f"{tnx}x{tny}", "pairs": pairs, "adam_steps": train_steps, "harvest_s": t_h,
                         "train_s": t_t, "loss_first": float(np.mean(hist[:20])),
                         "loss_last": float(np.mean(hist[-100:]))},
            "vs_fp64_gpu_pcg": v / fp64_value if fp64_value else None,
            "vs_multigrid_fcg": v / mg_value if mg_value else None,
            "note": "U-Net (4 levels, 16->128 channels, bf16, tcgen05 convolutions) after one V-cycle in each "
                    "flexible-CG preconditioner application; trained on the GPU by the project's kernels on pairs "
                    "from the method's own solves; FP64 true residual decides"}


def bench_learned2d(args, rank, world):
    """The learned preconditioner end to end at 512x256: training pairs harvested from
    seeded SIMP runs (vf uniform in [0.3, 0.6], point loads on the right edge, designs
    along the first iterations), the U-Net trained on the GPU (energy loss), then SIMP
    iterations of the MBB beam with the learned FCG, the multigrid FCG without the
    network, and the plain FP64 Jacobi PCG."""
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    import pansfem2_gb300 as P
    from pansfem2_gb300 import problems as PB
    P.load()
    nx, ny = args.nx or 512, args.ny or 256
    net, t_harvest, t_train, hist = harvest_and_train(nx, ny, args.pairs, args.train_steps, seed=rank)
    pr = PB.mbb_q4(nx, ny)
    res = {}
    clocks = None
    for solver in ("ir_learned_f32", "ir_mg_f32", "csr_jacobi_f64"):
        with P.Problem(pr) as prob, ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            prob.setup_bc()
            if solver == "ir_learned_f32":
                prob.attach_learned(net, pre_mg=True, nu_post=1)
            prob.simp_begin(solver=solver, cg_eps=args.eps, warm_start=solver != "csr_jacobi_f64")
            for _ in range(args.warmup):
                prob.simp_step()
            prob.sync()
            l0 = P.kernel_launches()
            t0 = time.perf_counter()
            infos = [prob.simp_step() for _ in range(args.steps)]
            clk.window(t0, time.perf_counter())
            nlaunch = P.kernel_launches() - l0
        if solver == "ir_learned_f32":
            clocks = clk.summary()
        t = sum(sum(i["phase_seconds"]) for i in infos)
        res[solver] = {"value": args.steps / t, "krylov_iterations": sum(i["solve"]["iterations"] for i in infos),
                       "kernel_launches": int(nlaunch),
                       "fell_back": sum(i["solve"]["fell_back"] for i in infos),
                       "true_residual_max": max(i["solve"]["rel_residual"] for i in infos), "f_last": infos[-1]["f"]}
    out = {"metric": learned_metric(nx, ny), "value": res["ir_learned_f32"]["value"], "unit": "SIMP iterations/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 / res["ir_learned_f32"]["value"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "bf16 network / f32 cycle / f64 FCG", "data": "synthetic",
           "config": {"workload": f"MBB half beam {nx}x{ny} Q4, MMA, R=3, vf=0.4; U-Net 4 levels 16->128",
                      "pairs": args.pairs, "train_steps": args.train_steps, "residual": f"FP64 relative {args.eps:g}"},
           "clocks": clocks, "gpu_launches": res["ir_learned_f32"]["kernel_launches"],
           "training": {"harvest_s": t_harvest, "train_s": t_train, "loss": "angle",
                        "loss_first": float(hist[:20].mean()), "loss_last": float(hist[-100:].mean())},
           "solvers": res,
           "learned_vs_fp64_pcg": res["ir_learned_f32"]["value"] / res["csr_jacobi_f64"]["value"],
           "learned_vs_multigrid": res["ir_learned_f32"]["value"] / res["ir_mg_f32"]["value"],
           "compliance_rel_diff_vs_fp64": abs(res["ir_learned_f32"]["f_last"] - res["csr_jacobi_f64"]["f_last"]) /
           abs(res["csr_jacobi_f64"]["f_last"])}
    print(json.dumps(out))


FEM_METRIC = "explicit-mesh system assemblies/s (element matrices, CSR pattern, values, loads)"


def fem_assembly_bytes(ne, nn, nfree, nnz, nen=4, nd=2, dim=2):
    """Algorithmic bytes per assembly kernel (FP64 values, int32 ids): the element kernel
    reads the connectivity, the coordinates and the moduli and writes the element matrices;
    the pattern kernel reads the node-to-element lists, the connectivity and the numbering and
    writes the row counts; the values kernel reads the element matrices once, the lists and the
    numbering and writes the CSR indices and values, F and the diagonal positions."""
    nk = nen * nd
    return {"element": ne * (4 * nen + 8 + 8 * nk * nk) + nn * dim * 8,
            "pattern": ne * nen * (4 + 4) + ne * nen * 4 + nn * (4 + 4 * nd) + nfree * 4,
            "values": ne * 8 * nk * nk + ne * nen * (4 + 4) + nn * (4 + 4 * nd) + nnz * 12 + nfree * 12}


def bench_fem(args, rank, world):
    """The general assembly path on an explicit mesh (1024x512 jittered Q4 plane strain with
    permuted node ids, 1.05M dofs, 18.9M stored entries): each step renumbers the dofs
    (SetDirichlet + Renumbering) and assembles the system from the coordinates (element
    matrices, CSR pattern, values, body force, tractions and point loads), as the reference
    does for every static analysis.  value: device time of the assembly kernels; e2e: the
    same calls with the moduli from host memory and the CSR system copied back to the host
    (psf_fem_get_system), the reference's form of the result; the CPU baseline is the
    oracle's assembly of the same mesh on one host core."""
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from pansfem2_gb300 import _lib
    from pansfem2_gb300 import fem as FM
    from pansfem2_gb300 import problems as PB
    nx, ny = args.nx or 1024, args.ny or 512
    m = PB.jittered_q4_mesh(nx, ny, seed=rank)
    fx = m["fixed"]
    ld = m["loads"]
    hb, hd = 0, 0
    with FM.FemMesh(0, m["coords"], m["conn"]) as mesh, ClockSampler(local) as clk:
        def step():
            mesh.set_dirichlet(fx[:, 0].astype(int), fx[:, 1].astype(int), fx[:, 2])
            mesh.set_loads(ld[:, 0].astype(int), ld[:, 1].astype(int), ld[:, 2])
            mesh.set_body_force(*m["body"])
            mesh.set_edge_loads(m["edges"], *m["traction"])
            mesh.assemble(m["E"], m["V"], m["t"])
            return mesh.timings()
        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        l0 = _lib.kernel_launches()
        t0 = time.perf_counter()
        ph = np.array([step() for _ in range(args.steps)])   # ms: element, pattern, values
        t_dev = time.perf_counter() - t0
        nlaunch = _lib.kernel_launches() - l0
        clk.window(t0, time.perf_counter())
        nfree, nnz = mesh.nfree, mesh.nnz
        # end to end: the same calls, the system copied back to host memory every step
        e2e_t = []
        for k in range(args.warmup + max(1, args.steps // 4)):
            t1 = time.perf_counter()
            step()
            sysm = mesh.system()
            if k >= args.warmup:
                e2e_t.append(time.perf_counter() - t1)
        hb = 8 * len(m["E"]) + fx.size * 4 + ld.size * 4 + m["edges"].size * 4
        hd = sum(a.nbytes for a in sysm)
    ms = ph.mean(0)
    dev_s, e2e_s = max_over_ranks([ms.sum() / 1e3, float(np.mean(e2e_t))], world)   # replicas: the slowest
    value = world / dev_s
    ne, nn = len(m["conn"]), len(m["coords"])
    by = fem_assembly_bytes(ne, nn, nfree, nnz)
    names = ["element", "pattern", "values"]
    k = int(np.argmax(ms))
    hbm, src = peaks()
    achieved = by[names[k]] / (ms[k] / 1e3) / 1e9
    tr = None
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as fh:
            tr = json.load(fh)[f"fem_{names[k]}"]["dram_bytes_per_launch"]
    except Exception:
        tr = None
    out = {"metric": FEM_METRIC, "value": value, "unit": "assemblies/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * dev_s, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"explicit Q4 plane-strain mesh {nx}x{ny}, jittered coordinates, permuted node "
                                  f"ids, body force + top-edge traction + point load",
                      "dofs": 2 * nn, "free_dofs": nfree, "stored_entries": nnz,
                      "l2": "inputs larger than L2 (element matrices 268 MB, CSR 227 MB)", "parallelism": f"replicas{world}"},
           "clocks": clk.summary(), "gpu_launches": int(nlaunch),
           "phases_ms": {n: float(v) for n, v in zip(names, ms)}, "wall_ms_per_step": 1e3 * t_dev / args.steps,
           "roofline": {"kernel": ["fem_ke_kernel", "pattern_count_kernel", "assemble_rows_kernel"][k],
                        "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                        "peak_source": src, "algorithmic_bytes": by[names[k]], "traffic": tr},
           "e2e": {"value": world / e2e_s, "unit": "assemblies/s", "h2d_bytes_per_step": int(hb),
                   "d2h_bytes_per_step": int(hd)}}
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import build as ob
        from oracle import pyoracle as O
        ob.build()
        nd = 2
        fixed = np.zeros(nn * nd, np.uint8)
        fixed[fx[:, 0].astype(int) * nd + fx[:, 1].astype(int)] = 1
        t1 = time.perf_counter()
        n2g, N = O.renumber(nn, nd, fixed)
        ip, ix, dat, F = O.assemble(0, m["conn"], m["coords"], m["E"], n2g, N, m["V"], m["t"], body=m["body"])
        F = O.neumann(F, ld[:, 0].astype(int), ld[:, 1].astype(int), ld[:, 2], nd, n2g)
        F = O.edge_loads(F, m["edges"], m["coords"], m["traction"], m["t"], n2g)
        tc = time.perf_counter() - t1
        same = bool(np.array_equal(ip, sysm[1]) and np.array_equal(ix, sysm[2]) and np.array_equal(dat, sysm[3])
                    and np.array_equal(F, sysm[4]))
        out["cpu_baseline"] = {"value": 1.0 / tc, "unit": "assemblies/s", "cores": 1, "kind": "port",
                               "sample": "one assembly of the same mesh by the oracle (numbering, element matrices, "
                                         "LIL rows, CSR, loads)",
                               "bitexact_vs_gpu": same}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def ncpus():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100, help="timed SIMP iterations (the MBB configuration runs 100)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--solver", default="ir_mg_f32")
    ap.add_argument("--baseline-solver", default=None,
                    help="plain FP64 GPU PCG: csr_jacobi_f64 (mbb2d) / ebe_jacobi_f64 (h8)")
    ap.add_argument("--no-compare", action="store_true", help="skip the plain FP64 GPU PCG comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-vtk", action="store_true", help="skip the VTK export of the final state")
    ap.add_argument("--no-learned", action="store_true", help="mbb2d: skip the learned-preconditioner block")
    ap.add_argument("--warm-start", type=int, default=1)
    ap.add_argument("--workload", default="mbb2d", choices=["mbb2d", "h8", "heat_batch", "c1", "learned2d", "fem_q4"])
    ap.add_argument("--pairs", type=int, default=4000, help="learned2d: training pairs")
    ap.add_argument("--train-steps", type=int, default=3000, help="learned2d: Adam steps")
    ap.add_argument("--instances", type=int, default=256, help="heat_batch: number of instances")
    ap.add_argument("--eps", type=float, default=1e-8, help="relative residual of every solve")
    ap.add_argument("--optimizer", default=None, choices=["oc", "mma", "conlin"],
                    help="mbb2d/h8: the optimiser (default: MMA for mbb2d, OC for h8)")
    ap.add_argument("--heaviside", action="store_true", help="mbb2d/h8: HeavisideFilter with beta continuation")
    ap.add_argument("--parity-iters", type=int, default=None,
                    help="mbb2d/h8/c1: SIMP iterations compared with the oracle and timed on the host "
                         "(default 3; 1 for h8)")
    ap.add_argument("--nx", type=int, default=None)
    ap.add_argument("--ny", type=int, default=None)
    ap.add_argument("--nz", type=int, default=None)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.workload == "heat_batch":
        return bench_heat_batch(args, rank, world)
    if args.workload == "learned2d":
        return bench_learned2d(args, rank, world)
    if args.workload == "fem_q4":
        return bench_fem(args, rank, world)
    pr, desc = workload(args.workload, args.nx, args.ny, args.nz)
    if args.optimizer is not None:   # the reference's other optimisers on the same problem
        pr["optimizer"] = {"oc": 0, "mma": 1, "conlin": 2}[args.optimizer]
        desc = desc.replace("MMA", args.optimizer.upper()).replace(", OC,", f", {args.optimizer.upper()},")
    if args.heaviside:   # HeavisideFilter with the samples' beta continuation (0.5, x2 every 40)
        pr.update(heaviside=1, beta=0.5, beta_every=40, beta_mult=2.0)
        desc += ", Heaviside projection (beta 0.5, x2 every 40 iterations)"
    from pansfem2_gb300 import problems as PB
    ne_w, nn_w, nd_w = PB.counts(pr)
    config = {"workload": desc, "dofs": nn_w * nd_w, "elements": ne_w,
              "residual": f"FP64 relative {args.eps:g}", "l2": "inputs larger than L2 (CSR 227 MB) for the FP64 path; "
              "FP32 matrix-free working set ~40 MB is L2-resident", "parallelism": f"replicas{world}"}

    parity_iters = args.parity_iters if args.parity_iters is not None else (1 if args.workload == "h8" else 3)
    if args.impl == "reference":
        if rank != 0:
            return
        # the steps actually timed: SIMP iterations 0 .. K-1 in full (a full CPU iteration at this
        # size takes tens of seconds, so K is bounded and reported as the step count)
        thr = ncpus()
        K = max(1, min(args.steps, parity_iters))
        orc, wall = oracle_first_iterations(pr, K, args.eps, thr)
        v = K / wall
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": K, "warmup": 0, "ms_per_step": 1e3 * wall / K, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "requested": {"steps": args.steps, "warmup": args.warmup,
                              "note": "the reference's iterations are timed from the uniform start without warm-up; "
                                      "the timed region is the whole run of K iterations"},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": thr, "kind": "port",
                                 "sample": cpu_sample_text(desc, K, args.eps, orc["cg_iters"], thr, wall)},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import pansfem2_gb300 as P
    P.load()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- value: device-resident design
    barrier()
    with ClockSampler(local) as clk:
        prob, infos, wall = run_device(pr, args.solver, args.warmup, args.steps, args.eps, bool(args.warm_start))
        clk.window(*prob.t_region)
    barrier()
    dev_t = sum(sum(i["phase_seconds"]) for i in infos)
    dev_t, = max_over_ranks([dev_t], world)
    value = world * args.steps / dev_t
    prob._sizes()
    ne, ndofs, nnz, nfree = prob.ne, prob.nnodes * prob.ndof, prob.nnz or 0, prob.nfree
    # ---- one VTK export of the final state (the samples' ExportToVTK.h file), outside the timed
    #      region: the call returns after the device work and the copy are queued; a host thread
    #      formats and writes the file
    vtk_info = None
    if not args.no_vtk and rank == 0:
        import tempfile
        try:
            with tempfile.TemporaryDirectory() as td:
                path = os.path.join(td, "state.vtk")
                t0 = time.perf_counter()
                prob.export_vtk(path, async_=True)
                t_call = time.perf_counter() - t0
                prob.export_wait()
                t_all = time.perf_counter() - t0
                vtk_info = {"call_ms": 1e3 * t_call, "file_ms": 1e3 * t_all, "bytes": os.path.getsize(path)}
        except Exception as e:   # reported, not fatal to the bench line
            vtk_info = {"error": str(e)[:200]}
    # ---- the reference's filter entry points on host arrays of this size (copies included),
    #      median of 5 calls each, outside the timed region
    entry_ms = None
    if rank == 0:
        try:
            s = prob.fields()["s"]
            prob.filter_setup()
            d = -np.abs(np.sin(np.arange(prob.ne) * 0.37)) - 0.1
            calls = {"DensityFilter.GetFilteredVariables": lambda: prob.filter_forward(s),
                     "DensityFilter.GetFilteredSensitivitis": lambda: prob.filter_backward(d),
                     "SensitivityFilter": lambda: prob.sensitivity_filter(s, d, 0),
                     "SensitivityFilter2": lambda: prob.sensitivity_filter(s, d, 1),
                     "HeavisideFilter.GetFilteredVariables": lambda: prob.heaviside_forward(4.0, s)}
            entry_ms = {}
            for name, fn in calls.items():
                fn()
                ts = []
                for _ in range(5):
                    t0 = time.perf_counter()
                    fn()
                    ts.append(1e3 * (time.perf_counter() - t0))
                entry_ms[name] = float(np.median(ts))
        except Exception as e:
            entry_ms = {"error": str(e)[:200]}
    prob.close()

    # roofline of the dominant kernel (the Krylov kernel)
    kit = sum(i["solve"]["iterations"] for i in infos)
    ksec = sum(i["solve"]["kernel_seconds"] for i in infos)
    klaunch = sum(i["solve"]["kernel_launches"] for i in infos)
    bpi = bytes_per_krylov_iteration(args.solver, pr, 18 * nfree, nfree)
    peak, peak_kind = peaks()
    achieved = bpi * kit / ksec / 1e9 if ksec > 0 else None
    # DRAM bytes per Krylov iteration from one ncu capture of the same kernel and workload
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(tpath) and klaunch > 0:
        try:
            t_it = json.load(open(tpath))[args.solver]["dram_bytes_per_iteration"]
            traffic = t_it * kit / klaunch
        except Exception:
            traffic = None

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * dev_t / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": ("f32 cycle / f32-pair Krylov / f64 true residual" if args.solver == "ir_mg_f32"
                     else "f32 inner / f64 refinement" if "f32" in args.solver else "f64"),
           "data": "synthetic (the MBB configuration; design starts uniform at vf)",
           "config": dict(config, solver=args.solver, warm_start=bool(args.warm_start)),
           "clocks": clk.summary(), "gpu_launches": None,
           "detail": {"wall_s": wall, "krylov_iterations": kit, "krylov_kernel_seconds": ksec,
                      "krylov_launches": klaunch, "f_last": infos[-1]["f"],
                      "true_residual_max": max(i["solve"]["rel_residual"] for i in infos),
                      "phase_seconds_mean": list(np.mean([i["phase_seconds"] for i in infos], axis=0))}}
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                       "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                       "kernel": KERNEL_NAME.get(args.solver, args.solver), "bytes_per_iteration": bpi,
                       "algorithmic_bytes_per_launch": bpi * kit / max(klaunch, 1),
                       "traffic_unit": "DRAM bytes per launch (read + write)",
                       "peak_source": peak_kind}
    # launches of our kernels in the timed region, counted by the library
    out["gpu_launches"] = int(prob.launches)

    if vtk_info is not None:
        out["vtk_export"] = vtk_info
    if entry_ms is not None:
        out["filter_entry_points_ms"] = entry_ms

    # ---- e2e through host buffers
    if not args.no_e2e:
        barrier()
        nsamp = min(10, args.steps)
        sample_at = sorted({(i * args.steps) // nsamp for i in range(nsamp)} | {args.steps - 1})
        einfos, ewall, h2d, d2h, designs = run_e2e(pr, args.solver, args.warmup, args.steps, args.eps,
                                                   bool(args.warm_start), sample_at=sample_at)
        barrier()
        ewall, = max_over_ranks([ewall], world)
        out["e2e"] = {"value": world * args.steps / ewall, "unit": UNIT, "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h}

    # ---- plain FP64 GPU PCG (the metric's denominator) at designs sampled evenly from the
    #      timed iterations.  That path cold-starts every solve, so one iteration's cost depends
    #      on its design only: the mean over the samples is its rate over the same iterations.
    if not args.no_compare:
        barrier()
        bsolver = args.baseline_solver or ("ebe_jacobi_f64" if args.workload == "h8" else "csr_jacobi_f64")
        args.baseline_solver = bsolver
        if args.no_e2e:   # the designs come from the host-buffer leg
            nsamp = min(10, args.steps)
            sample_at = sorted({(i * args.steps) // nsamp for i in range(nsamp)} | {args.steps - 1})
            _, _, _, _, designs = run_e2e(pr, args.solver, args.warmup, args.steps, args.eps,
                                          bool(args.warm_start), sample_at=sample_at)
        res = fp64_at_designs(pr, bsolver, designs, args.eps, first_iter=args.warmup)
        bt = float(np.mean([r["t"] for r in res.values()]))
        klast = max(res)
        out["fp64_gpu_pcg"] = {"solver": bsolver, "value": 1.0 / bt, "unit": UNIT,
                               "sampled_iterations": [args.warmup + k for k in sorted(res)],
                               "krylov_iterations_per_solve": float(np.mean([r["iters"] for r in res.values()])),
                               "speedup_of_value": value * bt,
                               "speedup_of_e2e": (out["e2e"]["value"] * bt) if "e2e" in out else None,
                               "f_at_last_sample": res[klast]["f"],
                               "compliance_rel_diff_at_samples": max(abs(res[k]["f"] - infos[k]["f"]) / abs(res[k]["f"])
                                                                     for k in res),
                               "note": "one SIMP iteration of the FP64 Jacobi PCG path (cold-started solve) from each "
                                       "sampled design of the timed trajectory; compliance compared with this "
                                       "solver's on the same design"}
        # split of the ratio: the same solvers with the other start (this solver cold-started at
        # every sampled design; the FP64 PCG warm-started at three of them, from the displacement
        # of one preceding iteration)
        cold = fp64_at_designs(pr, args.solver, designs, args.eps, first_iter=args.warmup, warm_start=False)
        t_cold = float(np.mean([r["t"] for r in cold.values()]))
        ks = sorted(designs)
        few = {k: designs[k] for k in sorted({ks[0], ks[len(ks) // 2], ks[-1]})}
        warm = fp64_at_designs(pr, bsolver, few, args.eps, first_iter=args.warmup, warm_start=True)
        t_warm = float(np.mean([r["t"] for r in warm.values()]))
        t_base_few = float(np.mean([res[k]["t"] for k in few]))
        out["ratio_split"] = {
            "this_solver_cold_start": {"value": 1.0 / t_cold, "unit": UNIT,
                                       "krylov_iterations_per_solve": float(np.mean([r["iters"] for r in cold.values()]))},
            "fp64_pcg_warm_start": {"value": 1.0 / t_warm, "unit": UNIT, "sampled_iterations": [args.warmup + k for k in few],
                                    "krylov_iterations_per_solve": float(np.mean([r["iters"] for r in warm.values()]))},
            "solver_gain_both_cold": bt / t_cold,
            "warm_start_gain_of_this_solver": t_cold / (dev_t / args.steps),
            "warm_start_gain_of_fp64_pcg": t_base_few / t_warm,
            "note": "value / fp64_gpu_pcg = solver_gain_both_cold x warm_start_gain_of_this_solver; the FP64 PCG "
                    "path itself cold-starts every solve (CG.h:423, x0 = 0)"}

    # ---- the learned preconditioner on the same window (rank 0)
    if rank == 0 and not args.no_learned and args.workload == "mbb2d":
        fp = out.get("fp64_gpu_pcg", {})
        out["learned"] = learned_leg(pr, pr["nx"], pr["ny"], args.warmup, args.steps, args.eps, fp.get("value"),
                                     fp.get("krylov_iterations_per_solve"), value)

    # ---- parity with the oracle at this size and the CPU baseline (rank 0 at N=1 only): the
    #      first K SIMP iterations from the uniform start, on the device (the product path, same
    #      solver and residual) and by the oracle on the host cores.  The oracle's run is timed
    #      whole and is the CPU baseline; its fields are the reference values of the parity check.
    if rank == 0 and world == 1 and not args.no_cpu:
        thr = ncpus()
        K = max(1, parity_iters)
        gpu = gpu_first_iterations(pr, args.solver, K, args.eps, bool(args.warm_start))
        orc, wall = oracle_first_iterations(pr, K, args.eps, thr)
        out["parity_vs_oracle"] = dict(parity_report(gpu, orc, K), residual=args.eps,
                                       note="device run (this solver, FP64 true residual <= eps) against the oracle "
                                            "(FP64 ScalingCG to the recurrence residual eps, sequential sums), "
                                            "iterations 0..K-1 from the uniform start")
        out["cpu_baseline"] = {"value": K / wall, "unit": UNIT, "cores": thr, "kind": "port",
                               "sample": cpu_sample_text(desc, K, args.eps, orc["cg_iters"], thr, wall)}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

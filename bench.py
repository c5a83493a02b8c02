"""Benchmark: time to |r|/|b| = 1e-10 for HISQ CG on 32^3x64 (mass 0.01).

One step = one block solve of N Gaussian even-site sources with the
production solver (FP16 or FP32 inner CG with FP64 reliable updates,
multi-source D_eo), inputs already resident in HBM.  The metric is seconds
per solved source (lower is better).  Reported beside it, measured in the
same run: the plain FP64 single-source GPU CG on the same sources, the D_eo
kernel's HBM roofline fraction (live CUDA-event timing of every launch in the
timed region), an end-to-end figure through the public C ABI with pinned host
buffers, and MILC's algorithm on the host cores (the C oracle port) on a
bounded sample of iterations.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIMS = (32, 32, 32, 64)
MASS = 0.01
RESID = 1e-10
LINK_A = 0.3
SEED_LINKS, SEED_SRC = 20251203, 4242
METRIC = "CG s to |r|/|b|=1e-10 per source (HISQ 32^3x64, m=0.01): mixed+multi-RHS; D_eo HBM GB/s"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def peaks():
    try:
        p = json.load(open(PEAKS))
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Sample nvidia-smi clocks during the timed region."""

    def __init__(self):
        self.samples, self.stop = [], threading.Event()

    def _run(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                      "--query-gpu=" + q, "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = max((float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # nvidia-smi prints "Active" / "Not Active" per reason
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > i + 2 and s[i + 2].strip() == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return rank, world


def max_over_ranks(value, world, device="cpu"):
    """The slowest rank's step time: the path has no data-path collective
    (one independent replica per GPU), only this timing reduction."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- reference arm
_CPU_CACHE = {}


def _cpu_problem():
    """The 32^3x64 HISQ problem on the host, built by the oracle library alone
    (the seeded generators of mks_synth.h are compiled into it), so that the
    reference arm never loads the product library."""
    from oracle import oracle as O
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    if _CPU_CACHE.get("dims") != DIMS:
        orc = O.Oracle(DIMS)
        U = orc.rephase(O.gen_thin_links(DIMS, SEED_LINKS, LINK_A))
        t0 = time.time()
        L = orc.hisq_links(U)
        _CPU_CACHE.update(dims=DIMS, orc=orc, fat=L["fat"][0], lng=L["lng"][0], t_links=time.time() - t0,
                          b=O.gen_vector(DIMS, SEED_SRC, O.EVEN))
    return _CPU_CACHE


def cpu_baseline(sample_iters=20, threads=None):
    """MILC's CG (the C oracle restatement of d_congrad5_fn_milc.c) on the host
    cores: time a bounded window of CG iterations on the full 32^3x64 HISQ
    problem (links built by the oracle too)."""
    threads = threads or os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    P = _cpu_problem()
    orc, fat, lng, b = P["orc"], P["fat"], P["lng"], P["b"]
    t0 = time.time()
    it, _, _ = orc.congrad(fat, lng, b, np.zeros_like(b), MASS, EVEN, 1e-30, 0.0, sample_iters, 1)
    dt = time.time() - t0
    return {"s_per_iter": dt / max(it, 1), "iters": it, "seconds": dt, "threads": threads,
            "link_build_s": P["t_links"]}


def cpu_full_solve(threads=None):
    """One complete FP64 solve of the first benchmark source to 1e-10 by the
    oracle's MILC CG on the host cores: its time (no extrapolation) and its
    solution, against which the GPU solution is checked."""
    threads = threads or os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    P = _cpu_problem()
    t0 = time.time()
    it, x, out = P["orc"].congrad(P["fat"], P["lng"], P["b"], np.zeros_like(P["b"]), MASS, EVEN, RESID, 0.0,
                                  1000, 10)
    return {"seconds": time.time() - t0, "iters": it, "x": x, "final_rsq": out[0], "threads": threads}


def cpu_extras(threads=None):
    """Labelled host-core timings of the other two workloads, oracle port of
    MILC's FP64 code: the 11-offset multi-shift CG on 32^3x64 (a bounded
    window of iterations, extrapolated to the FP64 GPU arm's iteration count)
    and the HISQ fermion force on 16^3x32 with 6 terms (one full call)."""
    from oracle import oracle as O
    threads = threads or os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    P = _cpu_problem()
    sig = 4 * MASS ** 2 + np.logspace(-4, 0, 11)
    window = 12
    t0 = time.time()
    it, _, _ = P["orc"].multicg_offset(P["fat"], P["lng"], P["b"], sig, EVEN, 1e-30, window, 1)
    dt = time.time() - t0
    ms = {"s_per_iter": dt / max(it, 1), "window_iters": it, "window_s": dt,
          "extrapolated_s_per_solve": dt / max(it, 1) * FP64_MULTISHIFT_ITERS_32C64,
          "sample": "%d iterations of MILC's 11-offset multi-shift CG (oracle port, FP64) on 32^3x64, "
                    "extrapolated to the FP64 GPU arm's %d iterations" % (it, FP64_MULTISHIFT_ITERS_32C64)}
    fdims = (16, 16, 16, 32)
    forc = O.Oracle(fdims)
    U = forc.rephase(O.gen_thin_links(fdims, 77, LINK_A))
    xxx = np.stack([O.gen_vector(fdims, 300 + j, O.EVENANDODD) for j in range(6)])
    t0 = time.time()
    forc.fermion_force_hisq(U, 0.01, np.linspace(0.1, 1.0, 6), xxx)
    force = {"s_per_call": time.time() - t0,
             "sample": "one HISQ fermion force call (oracle port of MILC's FP64 force, links smeared inside), "
                       "16^3x32, 6 terms"}
    return {"multishift_11_offsets_32c64": ms, "hisq_force_16c32_6terms": force, "threads": threads}


# dram__bytes_read.sum + dram__bytes_write.sum per launch of the multi-source
# D_eo family (mean of the plain D and the fused CG-epilogue launch), from
# ncu captures of this benchmark on GB300 (summaries under profiles/)
MEASURED_TRAFFIC = {
    ("single", 8, (32, 32, 32, 64), True): 0.5 * (1.614e9 + 2.095e9),
    # the plain D of the split-epilogue iteration (both D launches): mean of 8 launches
    ("single", 8, (32, 32, 32, 64), False): 1.6047e9,
}

# FP64 CG iterations to |r|/|b| = 1e-10 on this workload (32^3x64, m = 0.01,
# seeded links and source): MILC's CG and the GPU FP64 arm take the same
# count (identical recurrences), measured by the GPU arm on GB300.
FP64_ITERS_32C64 = 279
# the same for the FP64 11-offset multi-shift solve of the first source
FP64_MULTISHIFT_ITERS_32C64 = 277
EVEN, ODD, EVENANDODD = 0x02, 0x01, 0x03


def reference_arm(args):
    """MILC's FP64 CG (oracle port of d_congrad5_fn_milc.c) on the host cores.
    Loads only the oracle library: inputs come from the oracle's copy of the
    seeded generators.  A step is one bounded window of CG iterations on the
    full lattice; ms_per_step is the measured window time, and `value` the
    per-solve time extrapolated from the measured rate to the FP64 iteration
    count (labelled in cpu_baseline.sample)."""
    rank, world = dist_env()
    if rank != 0:
        return
    iters = args.ref_iters
    for _ in range(max(args.warmup, 1)):
        cpu_baseline(sample_iters=2)
    samples = [cpu_baseline(sample_iters=args.cpu_iters) for _ in range(max(args.steps, 1))]
    threads = samples[-1]["threads"]
    s_per_iter = sum(b["seconds"] for b in samples) / sum(b["iters"] for b in samples)
    window_ms = 1e3 * sum(b["seconds"] for b in samples) / len(samples)
    per_solve = s_per_iter * iters
    sample = ("%d windows of %d iterations of MILC's FEWSUMS CG on the full lattice (%.1f s measured, %.0f ms per "
              "window); value = measured s/iteration x %d iterations (extrapolated)"
              % (len(samples), args.cpu_iters, sum(b["seconds"] for b in samples), window_ms, iters))
    line = {"impl": "reference", "metric": METRIC, "value": per_solve, "unit": "s/solve", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": window_ms,
            "step": "one window of %d CG iterations (measured)" % args.cpu_iters,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded exp(i 0.3 H) thin links, HISQ smearing, Gaussian sources)",
            "config": {"workload": "HISQ CG 32^3x64 m=0.01 |r|/|b|=1e-10, single source, FP64",
                       "lattice": list(DIMS), "mass": MASS, "resid": RESID},
            "cpu_baseline": {"value": per_solve, "unit": "s/solve", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": per_solve, "unit": "s/solve", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_extras:
        line["extras"] = cpu_extras(threads)
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- extras
def nvtx_mark(torch, start):
    """Open (start=True) or close the NVTX range "timed_steps" around the
    timed launches, so that `ncu --nvtx --nvtx-include timed_steps/` profiles
    exactly them; a torch without NVTX support skips the marks."""
    try:
        if start:
            torch.cuda.nvtx.range_push("timed_steps")
        else:
            torch.cuda.nvtx.range_pop()
    except Exception:
        pass


def family_times(lib, _lib):
    fam = {}
    for name, k in _lib.KERNEL_FAMILIES.items():
        t, n = ctypes.c_double(), ctypes.c_longlong()
        lib.mks_timing_get(k, ctypes.byref(t), ctypes.byref(n))
        if n.value:
            fam[name] = {"ms": t.value, "launches": n.value}
    return fam


def force_chain(m, lib, _lib, torch):
    """The HISQ force workload on 16^3x32: a pseudofermion (Gaussian, even
    sites), its 6-term rational function (residues in [0.1, 1], offsets
    log-uniform in [1e-3, 1]) solved by the FP64 multi-shift to 1e-12, then
    the fermion force of the 6 solutions (the force call moves the solutions
    and momenta between host and device)."""
    fdims = (16, 16, 16, 32)
    m.set_lattice(fdims)
    V = int(np.prod(fdims))
    U = m.apply_phases(fdims, m.gen_thin_links(fdims, 77, LINK_A))
    m.load_hisq_links(U)
    rng = np.random.default_rng(4)
    residues = list(np.sort(rng.uniform(0.1, 1.0, 6)))
    offsets = np.logspace(-3, 0, 6)
    phi = torch.from_numpy(m.gen_vector(fdims, 4444, m.EVEN)).cuda()
    psim = [torch.zeros_like(phi) for _ in offsets]
    VP = ctypes.c_void_p * 6
    arg = _lib.InvertArg(2000, 5, m.EVEN, m.PREC_DOUBLE, 1e-12, 0.0, 0.1)
    res = (_lib.InvertResult * 6)()
    out = {}
    for rep in range(2):
        torch.cuda.synchronize()
        t0 = time.time()
        it = m.check(lib.mks_ks_multicg_offset_field_dev(phi.data_ptr(), VP(*[t.data_ptr() for t in psim]),
                                                         offsets.ctypes.data_as(_lib.DP), 6, 0, ctypes.byref(arg),
                                                         res), "force-chain multishift")
        torch.cuda.synchronize()
        t_solve = time.time() - t0
        xxx = []
        for t in psim:
            y = t.cpu().numpy().copy()
            y[V // 2:] = 0.0
            d = np.zeros_like(y)
            m.dslash_fn_field(y, d, m.ODD)
            y[V // 2:] = d[V // 2:]   # X on even sites, D_oe X on odd sites
            xxx.append(y)
        mom = np.zeros((V, 4, 10))
        t0 = time.time()
        m.eo_fermion_force_multi(0.02, residues, xxx, mom)
        t_force = time.time() - t0
        out = {"multishift_fp64_1e-12_s": t_solve, "multishift_iters": it, "force_s": t_force,
               "force_gflops_fp64": lib.mks_force_flops_last() / t_force / 1e9,
               "force_includes": "host<->device copies of 6 vectors and the momenta"}
    return out


def rhmc_2p1p1(m, dims, steps=10, tau=1.0):
    """The 2+1+1 HISQ RHMC trajectory (masses 0.0012 / 0.0363 / 0.432, the
    rational functions of milc_qcd_gb300/data, leapfrog, seeded exp(i 0.2 H)
    links), once with FP32 solves and force arithmetic and once all FP64
    from the same start: time per trajectory and Delta H of both."""
    from milc_qcd_gb300.rhmc import load_rhmc_params, update
    w = dict(RHMC_WORKLOAD)
    pfs = load_rhmc_params(os.path.join(ROOT, "milc_qcd_gb300", "data", w["rationals"]))
    n = len(pfs)
    m.set_lattice(dims)
    V = int(np.prod(dims))
    U0 = m.gen_thin_links(dims, w["seed"], 0.2)
    runs = {}
    for name, prec in (("f32", m.PREC_SINGLE), ("f64", m.PREC_DOUBLE)):
        m.gauge_load(U0)
        m.mom_load(np.zeros((V, 4, 10)))
        m.rng_seed(w["seed"])
        r = update(pfs, w["beta"], w["u0"], w["nflavors"], tau / steps, steps, "leapfrog",
                   [w["resid_md"]] * n, [w["resid_fa"]] * n, [w["resid_gr"]] * n, w["max_cg"], prec, prec, prec,
                   5, True, prec_force=prec)
        runs[name] = {k: r[k] for k in ("t_total", "t_solve", "t_fermion_force", "t_gauge_force", "t_links",
                                         "cg_iters", "n_solves", "unconverged", "delta_s")}
    return {"lattice": list(dims), "masses": [0.0012, 0.0363, 0.432], "pseudofermions": n, "steps": steps,
            "tau": tau, "integrator": "leapfrog", "poles": [p.MD.order for p in pfs], "runs": runs,
            "s_per_trajectory_f32": runs["f32"]["t_total"], "s_per_trajectory_f64": runs["f64"]["t_total"],
            "delta_h_f32_minus_f64": runs["f32"]["delta_s"] - runs["f64"]["delta_s"]}


def extras(m, lib, _lib, torch, srcs):
    """Figures for the other workloads of the same family, measured after the
    headline (not part of `value`): the multi-source sweep N = 1, 4, 8, 16
    (32^3x64, FP32 inner solve); the 11-offset multi-shift solve (32^3x64,
    sigma_i = 4m^2 + s_i, s_i log-uniform in [1e-4, 1]) in FP64 and mixed
    precision, with the rooflines of its update kernel and its D_eo pair; the
    HISQ force chain on 16^3x32 (6-term multi-shift to 1e-12, then the force);
    MILC's 2+1 RHMC regression set-up on 16^3x32; and the 2+1+1 RHMC
    trajectory on 48^3x96 in FP32 and FP64 from the same start (Delta H of
    both; MKS_BENCH_NO_48=1 leaves it out)."""
    out = {}
    sweep = {}
    for n in (1, 4, 8, 16):
        ss = [srcs[k % len(srcs)] * (1.0 + 0.01 * k) for k in range(n)]
        d_s = [torch.from_numpy(np.ascontiguousarray(s)).to("cuda") for s in ss]
        d_x = [torch.zeros_like(t) for t in d_s]
        arg = _lib.InvertArg(1000, 10, m.EVEN, m.PREC_SINGLE, RESID, 0.0, 0.1)
        res = (_lib.InvertResult * n)()
        VP = ctypes.c_void_p * n
        for rep in range(2):  # first run tunes and captures
            for t in d_x:
                t.zero_()
            torch.cuda.synchronize()
            t0 = time.time()
            m.check(lib.mks_ks_congrad_block_parity_dev(n, VP(*[t.data_ptr() for t in d_s]),
                                                        VP(*[t.data_ptr() for t in d_x]), MASS, 0,
                                                        ctypes.byref(arg), res), "sweep")
            torch.cuda.synchronize()
            dt = time.time() - t0
        sweep[str(n)] = {"s_per_solve": dt / n, "converged": all(res[k].converged for k in range(n))}
    out["multi_rhs_f32_s_per_solve"] = sweep
    sig = 4 * MASS ** 2 + np.logspace(-4, 0, 11)
    d_b = torch.from_numpy(srcs[0]).to("cuda")
    d_p = [torch.zeros_like(d_b) for _ in sig]
    VP = ctypes.c_void_p * len(sig)
    ms = {}
    Vh = int(np.prod(DIMS)) // 2
    peak, _ = peaks()
    for name, prec in (("f64", m.PREC_DOUBLE), ("single", m.PREC_SINGLE), ("half", m.PREC_HALF)):
        arg = _lib.InvertArg(1000, 10, m.EVEN, prec, RESID, 0.0, 0.1)
        res = (_lib.InvertResult * len(sig))()
        for rep in range(2):
            if rep == 1:
                lib.mks_timing_reset()
                lib.mks_timing_enable(1)
            torch.cuda.synchronize()
            t0 = time.time()
            it = m.check(lib.mks_ks_multicg_offset_field_dev(d_b.data_ptr(), VP(*[t.data_ptr() for t in d_p]),
                                                             sig.ctypes.data_as(_lib.DP), len(sig), 0,
                                                             ctypes.byref(arg), res), "multishift")
            torch.cuda.synchronize()
            dt = time.time() - t0
        lib.mks_timing_enable(0)
        fam = family_times(lib, _lib)
        ms[name] = {"s": dt, "iters": it, "max_final_rsq": max(res[k].final_rsq for k in range(len(sig))),
                    "converged": all(res[k].converged for k in range(len(sig))), "kernel_ms": fam}
        # rooflines of the multi-shift iteration's two kernels: the update
        # kernel (OpShiftUpdate) and the single-source D_eo pair
        n_it, n_upd = ctypes.c_longlong(), ctypes.c_longlong()
        lib.mks_multishift_counts(ctypes.byref(n_it), ctypes.byref(n_upd))
        # update-kernel vectors: r (read, write), ttt (read) and the lowest
        # shift's D_eo input (write) in the residual's precision; p_j and x_j
        # (read, write) of every shift advanced, in FP64 for targets below
        # 1e-7 (the library's choice unless MKS_MS_SHIFT64 forces one)
        vb = 48 if prec == m.PREC_DOUBLE else 24
        force64 = os.environ.get("MKS_MS_SHIFT64")
        vs = 48 if (prec == m.PREC_DOUBLE or (force64 != "0" and (force64 == "1" or RESID < 1e-7))) else 24
        if "shift" in fam and fam["shift"]["launches"]:
            upd_bytes = (4 * n_it.value * vb + 4 * n_upd.value * vs) * Vh
            gbs = upd_bytes / (fam["shift"]["ms"] * 1e-3) / 1e9
            ms[name]["roofline_shift_update"] = {
                "bytes": upd_bytes, "ms": fam["shift"]["ms"], "gbs": gbs, "frac": gbs / peak,
                "per_site": "4 vectors of %d B + 4 x shifts advanced vectors of %d B per iteration; %d iterations, "
                            "%d shift updates" % (vb, vs, n_it.value, n_upd.value)}
        dfam = {m.PREC_DOUBLE: "dslash_f64", m.PREC_SINGLE: "dslash_f32", m.PREC_HALF: "dslash_f16"}[prec]
        if prec != m.PREC_DOUBLE and dfam in fam and fam[dfam]["launches"]:
            # D pair per iteration: links twice (16 x 72 B FP32, 16 x 36 B FP16), input and output
            # vectors, and p and r of the fused epilogue (FP32); the reliable updates' FP64 D is
            # timed apart
            lk = 1152 if prec == m.PREC_SINGLE else 576
            vin = 24 if prec == m.PREC_SINGLE else 16
            pair = (2 * lk + (vin + vin) + (vin + 24 + 48)) * Vh
            d_ms = fam[dfam]["ms"] / (fam[dfam]["launches"] / 2)
            gbs = pair / (d_ms * 1e-3) / 1e9
            ms[name]["roofline_dslash_pair"] = {"bytes_per_pair": pair, "ms_per_pair": d_ms, "gbs": gbs,
                                                "frac": gbs / peak}
    out["multishift_11_offsets"] = ms
    out["force_chain_16c32_6terms"] = force_chain(m, lib, _lib, torch)
    out["rhmc_trajectory"] = rhmc_trajectory(m, RHMC_DIMS)
    if not os.environ.get("MKS_BENCH_NO_48"):
        out["rhmc_2p1p1_48c96"] = rhmc_2p1p1(m, (48, 48, 48, 96))
    m.set_lattice(DIMS)
    return out


# HISQ RHMC trajectory: MILC's 2+1 regression set-up (4 pseudofermion
# fields, the rational functions of MILC's sample rationals file, 3G1F,
# 10 steps of 0.02) on a larger seeded lattice, once with FP32 multi-shift
# solves and FP32 force arithmetic (the production setting) and once all
# FP64 from the same start, for Delta H against the FP64 run
RHMC_DIMS = (16, 16, 16, 32)


def rhmc_trajectory(m, dims, seed=5):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import rhmc_sample as R
    from milc_qcd_gb300.rhmc import update
    d = R.load()
    pfs = [dict(d["rational"][i], naik_term_epsilon=float(d["naik_eps"][i])) for i in range(R.N_PSEUDO)]
    m.set_lattice(dims)
    V = int(np.prod(dims))
    U0 = m.gen_thin_links(dims, seed, 0.2)
    out = {"lattice": list(dims), "pseudofermions": R.N_PSEUDO, "integrator": "3G1F", "steps": R.STEPS,
           "epsilon": R.EPSILON, "masses": [0.0018, 0.018], "rationals": "MILC sample (2+1, 4 fields)"}
    for name, prec in (("f32", m.PREC_SINGLE), ("f64", m.PREC_DOUBLE)):
        m.gauge_load(U0)
        m.mom_load(np.zeros((V, 4, 10)))
        m.rng_seed(seed)
        r = update(pfs, R.BETA, R.U0, R.nflavors(), R.EPSILON, R.STEPS, R.INT_ALG, R.RESID_MD, R.RESID_FA,
                   R.RESID_GR, R.MAX_CG, prec, prec, prec, R.NRESTART, True, prec_force=prec)
        out[name] = {"s_per_trajectory": r["t_total"], "delta_h": r["delta_s"], "cg_iters": r["cg_iters"],
                     "t_solve": r["t_solve"], "t_fermion_force": r["t_fermion_force"],
                     "t_gauge_force": r["t_gauge_force"], "t_links": r["t_links"], "unconverged": r["unconverged"]}
    out["delta_h_f32_minus_f64"] = out["f32"]["delta_h"] - out["f64"]["delta_h"]
    return out


# ---------------------------------------------------------------- GPU arm
def gpu_arm(args):
    import torch
    import milc_qcd_gb300 as m
    from milc_qcd_gb300 import _lib
    rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.cuda.current_device()
    lib = _lib.load()
    m.init(dev)
    m.set_lattice(DIMS)
    V = int(np.prod(DIMS))
    U = m.apply_phases(DIMS, m.gen_thin_links(DIMS, SEED_LINKS + rank, LINK_A))
    t0 = time.time()
    m.load_hisq_links(U)            # HISQ smearing on the GPU, FP64
    t_links = time.time() - t0
    del U
    N = args.nsrc
    prec = {"half": m.PREC_HALF, "single": m.PREC_SINGLE, "double": m.PREC_DOUBLE}[args.prec]
    srcs = [m.gen_vector(DIMS, SEED_SRC + 1000 * rank + k, m.EVEN) for k in range(N)]
    # device-resident inputs (MILC layout, FP64) for the `value` leg
    d_src = [torch.from_numpy(s).to("cuda") for s in srcs]
    d_dst = [torch.zeros_like(t) for t in d_src]
    arg = _lib.InvertArg(1000, 10, m.EVEN, prec, RESID, 0.0, 0.1)
    res = (_lib.InvertResult * N)()
    VP = ctypes.c_void_p * N

    def solve_dev():
        for t in d_dst:
            t.zero_()
        r = lib.mks_ks_congrad_block_parity_dev(N, VP(*[t.data_ptr() for t in d_src]),
                                                VP(*[t.data_ptr() for t in d_dst]), MASS, 0,
                                                ctypes.byref(arg), res)
        m.check(r, "block solve")
        return r

    # plain FP64 single-source GPU CG on the first source: the comparison arm
    arg64 = _lib.InvertArg(1000, 10, m.EVEN, m.PREC_DOUBLE, RESID, 0.0, 0.1)
    res64 = _lib.InvertResult()
    d64 = torch.zeros_like(d_src[0])
    for rep in range(2):  # the first call tunes the FP64 D_eo shape and captures the graphs
        d64.zero_()
        torch.cuda.synchronize()
        t0 = time.time()
        it64 = m.check(lib.mks_ks_congrad_parity_dev(d_src[0].data_ptr(), d64.data_ptr(), MASS, 0,
                                                     ctypes.byref(arg64), ctypes.byref(res64)), "fp64 solve")
        torch.cuda.synchronize()
        t_fp64 = time.time() - t0

    for _ in range(args.warmup):
        solve_dev()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches_before = lib.mks_launch_count()  # library kernels since mks_init (for ncu -s)
    launches0 = lib.mks_launch_count()
    stream = torch.cuda.ExternalStream(lib.mks_stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters = []
    with Clocks() as clk:
        torch.cuda.synchronize()
        nvtx_mark(torch, True)
        ev0.record(stream)
        for _ in range(args.steps):
            iters.append(solve_dev())
        ev1.record(stream)
        torch.cuda.synchronize()
        nvtx_mark(torch, False)
    launches = lib.mks_launch_count() - launches0
    step_ms = ev0.elapsed_time(ev1) / args.steps
    step_ms = max_over_ranks(step_ms, world, "cuda")
    # Kernel times (kernel_ms, roofline): the same steps once more with a CUDA
    # event pair recorded around every library launch on the library's stream.
    # The event records add gaps between launches (3-4 % of the step), so
    # `value` comes from the pass above, which records none.
    lib.mks_timing_reset()
    lib.mks_timing_enable(1)
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev2.record(stream)
    for _ in range(args.steps):
        solve_dev()
    ev3.record(stream)
    torch.cuda.synchronize()
    lib.mks_timing_enable(0)
    step_ms_timed = ev2.elapsed_time(ev3) / args.steps
    per_src = step_ms / 1e3 / N
    reliable = [res[k].reliable_updates for k in range(N)]
    # verify every solution in FP64 on the GPU: r = b - M^dag M x with the FP64 operator
    x_host = [t.cpu().numpy() for t in d_dst]
    final_rsq = max(res[k].final_rsq for k in range(N))
    converged = all(res[k].converged for k in range(N))
    sum_iters = sum(res[k].final_iters for k in range(N))
    # sustained solver rate in MILC's count (1187 flop per site per CG
    # iteration, d_congrad5_fn_milc.c:82)
    cg_gflops = 1187.0 * (V // 2) * sum_iters / (step_ms * 1e-3) / 1e9
    # kernel roofline: the sloppy D_eo (dominant kernel), live CUDA-event timing
    fam = {m.PREC_HALF: 2, m.PREC_SINGLE: 1, m.PREC_DOUBLE: 0}[prec]
    if N > 1 and prec != m.PREC_DOUBLE:
        fam = 3
    kernel_ms = {}
    for name, k in _lib.KERNEL_FAMILIES.items():
        t, n = ctypes.c_double(), ctypes.c_longlong()
        lib.mks_timing_get(k, ctypes.byref(t), ctypes.byref(n))
        if n.value:
            kernel_ms[name] = {"ms_per_step": t.value / args.steps, "launches_per_step": n.value / args.steps}
    tot_ms, nl = ctypes.c_double(), ctypes.c_longlong()
    lib.mks_timing_get(fam, ctypes.byref(tot_ms), ctypes.byref(nl))
    # launch shapes the autotuner chose for the sloppy D_eo of this solve
    shapes = {}
    G, nb, blk, tma = (ctypes.c_int() for _ in range(4))
    def variant(v):
        if v is None or v < 0:
            return None
        kind = ["direct loads", "TMA-staged links", "direct loads, pipelined",
                "cp.async link buffers x%d" % (v >> 3)][v & 3]
        return kind + (", persistent grid" if v & 4 else "")
    if lib.mks_tuned_shape(prec, N, ctypes.byref(G), ctypes.byref(nb), ctypes.byref(blk)) == 0:
        shapes["D"] = {"G": G.value, "NB": nb.value, "block": blk.value,
                       "kernel": variant(lib.mks_tuned_variant(prec, N, 0))}
    if lib.mks_tuned_shape_epi(prec, N, ctypes.byref(G), ctypes.byref(nb), ctypes.byref(blk),
                               ctypes.byref(tma)) == 0:
        shapes["D+epilogue"] = {"G": G.value, "NB": nb.value, "block": blk.value, "tma": tma.value,
                                "kernel": variant(lib.mks_tuned_variant(prec, N, 1))}
    # Launches that did work: a batch of iterations replayed as a graph stops
    # early (its remaining kernels return at once) when a source asks for a
    # reliable update, so the launch count includes such empty launches.  The
    # block runs as many CG iterations as its slowest source, two D_eo each
    # (final_iters counts the CG iterations, the initial true residual and
    # the reliable updates).
    cg_iters = max(res[k].final_iters - 1 - res[k].reliable_updates for k in range(N))
    d_executed = 2 * cg_iters * args.steps if N > 1 and prec != m.PREC_DOUBLE else nl.value
    dslash_ms = tot_ms.value / max(d_executed, 1)
    Vh = V // 2
    # the second D of an iteration carries the fused CG epilogue unless the
    # epilogue runs as its own kernel (then no fused-epilogue shape was tuned)
    fused = lib.mks_tuned_shape_epi(prec, N, None, None, None, None) == 0
    if prec == m.PREC_HALF:
        # K1: half links + half in/out (+norms); K2: half links + half in, f32 out, f32 p and r read
        per_site = 16 * 18 * 2 + N * 0.5 * ((16 + 16) + (16 + 24 + 24 + 24))
    elif prec == m.PREC_SINGLE:
        per_site = 16 * 18 * 4 + N * (0.5 * ((24 + 24) + (24 + 24 + 24 + 24)) if fused else (24 + 24))
    else:
        per_site = 16 * 18 * 8 + N * 0.5 * ((48 + 48) + (48 + 48 + 48 + 48))
    alg_bytes = per_site * Vh
    traffic = MEASURED_TRAFFIC.get((args.prec, N, tuple(DIMS), fused))
    peak, peak_kind = peaks()
    achieved = alg_bytes / (dslash_ms * 1e-3) / 1e9
    # plain FP64 D_eo and FP32 D_eo standalone timings (L2 flushed between launches)
    ms64, ms32 = ctypes.c_double(), ctypes.c_double()
    m.check(lib.mks_bench_dslash(m.PREC_DOUBLE, 1, m.EVEN, 0, 10, 1, ctypes.byref(ms64)), "bench64")
    m.check(lib.mks_bench_dslash(m.PREC_SINGLE, 1, m.EVEN, 0, 10, 1, ctypes.byref(ms32)), "bench32")
    gbs32 = 1200.0 * Vh / (ms32.value * 1e-3) / 1e9

    # e2e: the same solve through the host-array C ABI from page-locked buffers; the
    # library's layout kernels read the sources and guesses and write the solutions
    # over the host link inside the timed region (the parity halves counted below).
    # Each step gets its own zero initial guess, prepared before the clock starts.
    e2e_steps = max(1, args.steps)
    h_src = [torch.from_numpy(s).pin_memory() for s in srcs]
    h_dst = [[torch.zeros_like(t).pin_memory() for t in h_src] for _ in range(e2e_steps)]
    DPv = _lib.DP * N
    psrc = DPv(*[ctypes.cast(t.data_ptr(), _lib.DP) for t in h_src])
    pdst = [DPv(*[ctypes.cast(t.data_ptr(), _lib.DP) for t in h_dst[k]]) for k in range(e2e_steps)]
    torch.cuda.synchronize()
    t0 = time.time()
    for k in range(e2e_steps):
        m.check(lib.mks_ks_congrad_block_parity(N, psrc, pdst[k], MASS, 0, ctypes.byref(arg), res), "e2e solve")
    torch.cuda.synchronize()
    e2e_per_src = (time.time() - t0) / e2e_steps / N
    bytes_field = V * 6 * 8

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": per_src, "unit": "s/solve", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": {"half": "f16/f32+f64", "single": "f32+f64", "double": "f64"}[args.prec],
        "data": "synthetic (seeded exp(i 0.3 H) thin links, HISQ smearing on GPU, Gaussian even-site sources)",
        "config": {"workload": "HISQ CG 32^3x64 m=0.01 |r|/|b|=1e-10, block of %d sources, %s inner solve, "
                               "FP64 reliable updates (delta=0.1)" % (N, args.prec),
                   "lattice": list(DIMS), "mass": MASS, "resid": RESID, "nsrc": N, "inner": args.prec,
                   "l2": "inputs larger than L2 (links alone 0.6-2.4 GB)"},
        "fp64_plain_single_rhs": {"s_per_solve": t_fp64, "iters": it64, "final_rsq": res64.final_rsq},
        "speedup_vs_fp64_plain": t_fp64 / per_src,
        "iters": iters, "reliable_updates": reliable, "final_rsq_max": final_rsq, "converged": converged,
        "cg_gflops": cg_gflops,
        "dslash_gbs": {"f32_single_rhs": gbs32, "f32_ms": ms32.value, "f64_ms": ms64.value,
                       "f64_gflops": 1146.0 * Vh / (ms64.value * 1e-3) / 1e9},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_unit": "bytes per launch (ncu DRAM read + write)",
                     "kernel": "k_dslash (%s, nsrc=%d%s)" % (args.prec, N, "" if fused else ", plain D pair"),
                     "peak_source": peak_kind, "avg_launch_ms": dslash_ms, "algorithmic_bytes_per_launch": alg_bytes,
                     "launches_executed": d_executed, "launches_issued": nl.value},
        # the C ABI moves the solved parity's half of each field: source and
        # initial guess in, solution out
        "e2e": {"value": e2e_per_src, "unit": "s/solve", "h2d_bytes_per_step": N * bytes_field,
                "d2h_bytes_per_step": N * bytes_field // 2},
        "gpu_launches": int(launches),
        "launches_before_timed": int(launches_before),
        "kernel_ms": kernel_ms,
        "kernel_timing_pass": {"ms_per_step": step_ms_timed,
                               "how": "a second pass of the same steps with a CUDA event pair around every "
                                      "library launch; kernel_ms and roofline come from it, value from the "
                                      "first pass"},
        "dslash_shapes": shapes,
        "clocks": clk.summary(),
        "link_build_s": t_links,
    }
    if not args.no_extras:
        line["extras"] = extras(m, lib, _lib, torch, srcs)
    if not args.no_cpu and world == 1:
        # the oracle (MILC's FP64 CG restated in C) solves the first source
        # completely on the host cores: a full-solve CPU time, and the
        # reference solution for the GPU's; every GPU solution's true residual
        # is recomputed with the oracle's D (its own links, built on the host)
        full = cpu_full_solve()
        line["cpu_baseline"] = {"value": full["seconds"], "unit": "s/solve", "cores": full["threads"],
                                "kind": "port",
                                "sample": "one complete FP64 solve of the first source to 1e-10 by the oracle port "
                                          "of MILC's CG (%d iterations, no extrapolation)" % full["iters"]}
        line["oracle_check"] = oracle_check(x_host, srcs, full)
    print(json.dumps(line), flush=True)


def oracle_check(x_host, srcs, full):
    """Each GPU solution against the oracle: the FP64 true residual
    |b - (4m^2 - D_eo D_oe) x| / |b| recomputed with the oracle's D for every
    source, and the relative solution error against the oracle's full FP64 CG
    solve of the first source."""
    P = _cpu_problem()
    orc, fat, lng = P["orc"], P["fat"], P["lng"]
    Vh = srcs[0].shape[0] // 2
    res = []
    for x, b in zip(x_host, srcs):
        Dx = orc.dslash(fat, lng, orc.dslash(fat, lng, x, ODD), EVEN)
        r = b[:Vh] - (4 * MASS ** 2 * x[:Vh] - Dx[:Vh])
        res.append(float(np.linalg.norm(r) / np.linalg.norm(b[:Vh])))
    xo = full["x"][:Vh]
    return {"true_residual_by_oracle_D": res,
            "solution_rel_error_vs_oracle_cg_src0": float(np.linalg.norm(x_host[0][:Vh] - xo) / np.linalg.norm(xo)),
            "oracle_cg_iters_src0": full["iters"],
            "links": "GPU HISQ smearing (solve) vs oracle HISQ smearing (check), same seeded thin links"}


# 2+1+1 HISQ RHMC trajectory (the molecular-dynamics workload): 48^3x96,
# masses 0.0012 / 0.0363 / 0.432 (rational functions generated by
# milc_qcd_gb300/data/make_rationals.py), links from seeded exp(i 0.2 H),
# 10 leapfrog steps, tau = 1; once with FP32 solves and force arithmetic
# and once all FP64 from the same start (Delta H against the FP64 run).
RHMC_WORKLOAD = dict(dims=(48, 48, 48, 96), beta=6.3, u0=0.86, nflavors=4, steps=10, tau=1.0,
                     rationals="rationals.hisq_2p1p1_ml0.0012_ms0.0363_mc0.432.txt",
                     resid_md=1e-6, resid_fa=1e-10, resid_gr=1e-10, max_cg=5000, seed=7)


def rhmc_workload(args):
    import milc_qcd_gb300 as m
    from milc_qcd_gb300.rhmc import load_rhmc_params, update
    w = dict(RHMC_WORKLOAD)
    if args.dims:
        w["dims"] = tuple(args.dims)
    dims = w["dims"]
    pfs = load_rhmc_params(os.path.join(ROOT, "milc_qcd_gb300", "data", w["rationals"]))
    n = len(pfs)
    m.init(0)
    m.set_lattice(dims)
    V = int(np.prod(dims))
    U0 = m.gen_thin_links(dims, w["seed"], 0.2)
    runs = {}
    with Clocks() as clk:
        for name, prec in (("f32", m.PREC_SINGLE), ("f64", m.PREC_DOUBLE)):
            m.gauge_load(U0)
            m.mom_load(np.zeros((V, 4, 10)))
            m.rng_seed(w["seed"])
            r = update(pfs, w["beta"], w["u0"], w["nflavors"], w["tau"] / w["steps"], w["steps"], "leapfrog",
                       [w["resid_md"]] * n, [w["resid_fa"]] * n, [w["resid_gr"]] * n, w["max_cg"], prec, prec, prec,
                       5, True, prec_force=prec)
            runs[name] = {k: r[k] for k in ("t_total", "t_solve", "t_fermion_force", "t_gauge_force", "t_links",
                                             "cg_iters", "n_solves", "unconverged", "delta_s", "start", "end")}
    line = {"metric": "RHMC s per trajectory (2+1+1 HISQ, %s)" % "x".join(map(str, dims)),
            "value": runs["f32"]["t_total"], "unit": "s/trajectory", "n_gpus": 1, "steps": 1, "warmup": 0,
            "higher_is_better": False, "dtype": "f32+f64", "data": "synthetic (seeded exp(i 0.2 H) links)",
            "config": {"workload": "2+1+1 HISQ RHMC trajectory, leapfrog 10 steps, tau 1", "lattice": list(dims),
                       "masses": [0.0012, 0.0363, 0.432], "beta": w["beta"], "u0": w["u0"],
                       "pseudofermions": n, "poles": [p.MD.order for p in pfs],
                       "resid_md_fa_gr": [w["resid_md"], w["resid_fa"], w["resid_gr"]]},
            "delta_h_f32": runs["f32"]["delta_s"], "delta_h_f64": runs["f64"]["delta_s"],
            "delta_h_f32_minus_f64": runs["f32"]["delta_s"] - runs["f64"]["delta_s"],
            "runs": runs, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


# HISQ link rebuild + fermion force of one molecular-dynamics step of the
# 2+1+1 workload: 38 rational-function terms (16 light + 12 strange in the
# eps = 0 Naik group, 10 charm in the eps_naik(0.432) group), seeded
# synthetic links and solutions; once in FP64 and once in the FP32 setting.
def force_workload(args):
    import milc_qcd_gb300 as m
    from milc_qcd_gb300.remez import eps_naik
    dims = tuple(args.dims) if args.dims else (48, 48, 48, 96)
    V = int(np.prod(dims))
    m.init(0)
    m.set_lattice(dims)
    lib = m._lib.load()
    m.gauge_load(m.gen_thin_links(dims, 7, 0.2))
    eps = (0.0, eps_naik(0.432))
    rng = np.random.default_rng(3)
    nterms, orders = 38, [28, 10]
    xxx = [rng.standard_normal((V, 6)) for _ in range(nterms)]
    res = rng.uniform(0.01, 0.1, nterms)
    mom = np.zeros((V, 4, 10))
    out = {}
    runs = {"both": (("f64", m.PREC_DOUBLE), ("f32", m.PREC_SINGLE)), "double": (("f64", m.PREC_DOUBLE),),
            "single": (("f32", m.PREC_SINGLE),)}[args.md_prec]
    for name, prec in runs:
        m.md_precision(prec)
        per = []
        for rep_ in range(max(args.warmup, 0) + max(args.steps, 1)):
            lib.mks_timing_reset()
            lib.mks_timing_enable(1)
            t0 = time.time()
            m.rebuild_links("hisq", eps)
            t1 = time.time()
            m.eo_fermion_force_multi(0.1, res, xxx, mom, n_orders_naik=orders, n_naiks=2)
            t2 = time.time()
            lib.mks_timing_enable(0)
            fam = {}
            for fname, k in m._lib.KERNEL_FAMILIES.items():
                t, n = ctypes.c_double(), ctypes.c_longlong()
                lib.mks_timing_get(k, ctypes.byref(t), ctypes.byref(n))
                if n.value:
                    fam[fname] = {"ms": t.value, "launches": n.value}
            per.append({"links_s": t1 - t0, "force_s_incl_host_copies": t2 - t1, "kernel": fam})
        out[name] = per[-1]
    m.md_precision(m.PREC_DOUBLE)
    line = {"metric": "HISQ link rebuild + fermion force, s per molecular-dynamics step (%s)" % "x".join(map(str, dims)),
            "value": sum(out[k]["links_s"] + out[k]["force_s_incl_host_copies"] for k in list(out)[-1:]),
            "unit": "s/step", "n_gpus": 1,
            "higher_is_better": False, "dtype": "f32+f64", "data": "synthetic (seeded exp(i 0.2 H) links, Gaussian solutions)",
            "config": {"workload": "HISQ links (2 Naik groups) + fermion force, 38 terms", "lattice": list(dims)},
            "runs": out}
    print(json.dumps(line), flush=True)


# The 11-offset multi-shift alone (32^3x64, sigma_i = 4m^2 + s_i, s_i
# log-uniform in [1e-4, 1], to 1e-10; --prec selects the sloppy precision):
# one warm solve, one timed solve without per-launch events (with its
# launch counts, for an ncu launch list of exactly that solve), then one
# with per-launch CUDA events for the kernel families.
def multishift_workload(args):
    import torch
    import milc_qcd_gb300 as m
    from milc_qcd_gb300 import _lib
    lib = _lib.load()
    m.init(0)
    m.set_lattice(DIMS)
    m.load_hisq_links(m.apply_phases(DIMS, m.gen_thin_links(DIMS, SEED_LINKS, LINK_A)))
    prec = {"half": m.PREC_HALF, "single": m.PREC_SINGLE, "double": m.PREC_DOUBLE}[args.prec]
    sig = 4 * MASS ** 2 + np.logspace(-4, 0, 11)
    d_b = torch.from_numpy(m.gen_vector(DIMS, SEED_SRC, m.EVEN)).to("cuda")
    d_p = [torch.zeros_like(d_b) for _ in sig]
    VP = ctypes.c_void_p * len(sig)
    arg = _lib.InvertArg(1000, 10, m.EVEN, prec, RESID, 0.0, 0.1)
    res = (_lib.InvertResult * len(sig))()
    stream = torch.cuda.ExternalStream(lib.mks_stream())

    def solve():
        return m.check(lib.mks_ks_multicg_offset_field_dev(d_b.data_ptr(), VP(*[t.data_ptr() for t in d_p]),
                                                           sig.ctypes.data_as(_lib.DP), len(sig), 0,
                                                           ctypes.byref(arg), res), "multishift")
    solve()
    torch.cuda.synchronize()
    launches_before = lib.mks_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nvtx_mark(torch, True)
    ev0.record(stream)
    it = solve()
    ev1.record(stream)
    torch.cuda.synchronize()
    nvtx_mark(torch, False)
    launches = lib.mks_launch_count() - launches_before
    lib.mks_timing_reset()
    lib.mks_timing_enable(1)
    solve()
    torch.cuda.synchronize()
    lib.mks_timing_enable(0)
    line = {"metric": "11-offset multi-shift CG s per solve (HISQ %s, m=0.01, 1e-10)" % "x".join(map(str, DIMS)),
            "value": ev0.elapsed_time(ev1) / 1e3, "unit": "s/solve", "n_gpus": 1, "higher_is_better": False,
            "dtype": {"half": "f16/f32+f64", "single": "f32+f64", "double": "f64"}[args.prec],
            "data": "synthetic (seeded exp(i 0.3 H) thin links, HISQ smearing on GPU, Gaussian source)",
            "iters": it, "max_final_rsq": max(r.final_rsq for r in res),
            "converged": all(r.converged for r in res), "gpu_launches": int(launches),
            "launches_before_timed": int(launches_before), "kernel_ms": family_times(lib, _lib)}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    # defaults: the fastest measured configuration per solved source on GB300
    ap.add_argument("--nsrc", type=int, default=8)
    # a smaller lattice for profiling captures (the metric is quoted on 32^3x64)
    ap.add_argument("--dims", type=int, nargs=4, default=None)
    ap.add_argument("--prec", default="single", choices=["half", "single", "double"])
    ap.add_argument("--cpu-iters", type=int, default=12)
    ap.add_argument("--ref-iters", type=int, default=int(os.environ.get("MKS_REF_ITERS", "0")) or None)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--md-prec", default="both", choices=["both", "single", "double"],
                    help="force workload: the molecular-dynamics precisions to run")
    ap.add_argument("--workload", default="cg", choices=["cg", "rhmc", "force", "multishift"],
                    help="cg: the headline CG benchmark; rhmc: one 2+1+1 HISQ RHMC trajectory; "
                         "force: HISQ link rebuild + fermion force of one molecular-dynamics step; "
                         "multishift: the 11-offset multi-shift solve alone")
    args = ap.parse_args()
    if args.dims:
        global DIMS
        DIMS = tuple(args.dims)
    if args.workload in ("rhmc", "force", "multishift"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the %s workload has no CPU reference arm"
                              % args.workload}))
            return
        {"rhmc": rhmc_workload, "force": force_workload, "multishift": multishift_workload}[args.workload](args)
        return
    if args.impl == "reference":
        if args.ref_iters is None:
            args.ref_iters = FP64_ITERS_32C64
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()

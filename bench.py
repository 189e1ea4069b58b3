#!/usr/bin/env python
"""RCCD s/iter and TFLOP/s at nbf=200 on one GB300: split precision vs FP64.

Workload: the seeded synthetic closed-shell system nbf=200, nocc=40, nvir=160, naux=600
(B-factored AO integrals, 12.8 GB).  A "step" is one RCCD sweep (all intermediates, the T2
update, the energy and the DIIS extrapolation) with the integrals resident in HBM.

The split form timed here is the library's default split setting (JUES_PREC_SPLIT): integral
blocks from the three-plane transform, CC sweeps on two planes (FP16 integer digits on the
tcgen05 tensor cores, FP32 accumulation, FP64 everywhere else).  Its converged energy error
against the FP64 oracle is reported for the same setting.

Arms:
  default            libjuesgpu.so: split sweeps timed with CUDA events on the library's stream;
                     one FP64 sweep beside them; converged energy errors against the FP64 golden;
                     e2e = one converged mRCCD.do_rccd C-ABI call with host buffers.
  --impl reference   the CPU restatement of the reference's RCCD.jl sweep on all host cores, cut
                     into 16 stages of real work per sweep (one stage per step).

Under torchrun (N > 1) every rank runs an independent replica on its own GPU (the path has no
data-parallel split of one system); rank 0 prints max-over-ranks timing.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "jues.jl_gb300")]

import numpy as np  # noqa: E402

METRIC = "RCCD s/iter & TFLOP/s at nbf=200: split-BF16 vs FP64 on 1 GB300 at ≤1 µEh"
SHAPES = {"S200": ("S200", 200, 40, 600), "S100": ("S100", 100, 20, 300)}
SHAPE = SHAPES["S200"]
SPLIT_DTYPE = "fp16-int split (2 planes sweeps, 3 planes integrals; fp32 acc) + f64"
# GB300 FP64 peak as published by NVIDIA (a specification figure, not measured on this machine)
FP64_SPEC_TFLOPS = 1.25


def ccd_ref_flops(o, v):
    """The reference's GEMM set per sweep (mRCCD.jl): 4o^2v^4+16o^3v^3+4o^4v^2+6o^2v^3+6o^3v^2."""
    o, v = float(o), float(v)
    return 4 * o**2 * v**4 + 16 * o**3 * v**3 + 4 * o**4 * v**2 + 6 * o**2 * v**3 + 6 * o**3 * v**2


def ccd_exec_flops(o, v):
    """Contractions this library executes per sweep (Wabef never formed, Fmi in the ladder)."""
    o, v = float(o), float(v)
    return 2 * o**2 * v**4 + 12 * o**3 * v**3 + 4 * o**4 * v**2 + 4 * o**2 * v**3 + 2 * o**3 * v**2


def folds(o, v):
    """Whether the split sweeps run the folded ladders (nocc <= 64 and nvir <= 361)."""
    return o <= 64 and v * (v + 1) // 2 <= 65536 - 64


def ccd_split_gemm_flops(o, v):
    """One product's flops per CCD split sweep of each tcgen05 GEMM scope (3 products run): X and
    the ladders folded over the pairs (i <= j), (a <= b) when folds(o, v), and the K-stacked rings."""
    ov = float(o * v)
    if folds(o, v):
        np_, nq = o * (o + 1) / 2.0, v * (v + 1) / 2.0
        x, lad = 2 * 2.0 * o * o * np_ * nq, 2 * 2.0 * np_ * nq * (np_ + nq)
    else:
        x, lad = 2.0 * o**4 * v**2, 2.0 * o**2 * v**2 * (o**2 + v**2)
    return {"ccd_x": x, "ccd_pp_ladder": lad, "ccd_wj": 4 * ov**3, "ccd_wk": 2 * ov**3, "ccd_ring": 6 * ov**3}


def ladder_launch_flops(o, v):
    """Executed (3-product) flops of one ladder GEMM launch: one folded sign, or the whole ladder."""
    if folds(o, v):
        np_, nq = o * (o + 1) / 2.0, v * (v + 1) / 2.0
        return 3 * 2.0 * np_ * nq * (np_ + nq)
    return 3 * 2.0 * o**2 * v**2 * (v**2 + o**2)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def ready(self, timeout=5.0):
        """Wait for nvidia-smi's first line (its start-up takes ~0.1 s), then drop it, so the
        samples kept are the ones taken during the timed region that follows."""
        t = time.perf_counter()
        while self.proc and not self.lines and time.perf_counter() - t < timeout:
            time.sleep(0.01)
        self.lines.clear()

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(gpus):
    """Replica setup (juesgpu.replicas): NCCL process group under torchrun, none for one GPU."""
    from juesgpu import replicas
    r = replicas.setup()
    return r.world_size, r.rank, r.local_rank, (r if r.world_size > 1 else None)


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    return x if pg is None else pg.max(x)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p, "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def load_traffic():
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def golden(name):
    try:
        with open(os.path.join(ROOT, "tests", "golden", "synthetic_golden.json")) as f:
            return json.load(f).get(name, {})
    except OSError:
        return {}


def blas_threads():
    """Threads numpy's BLAS runs with (the library numpy links, queried directly)."""
    try:
        from threadpoolctl import threadpool_info
        for d in threadpool_info():
            if d.get("user_api") == "blas":
                return {"library": d.get("internal_api"), "threads": d.get("num_threads")}
    except ImportError:
        pass
    try:
        paths = sorted({ln.split()[-1] for ln in open("/proc/self/maps") if "openblas" in ln.lower()
                        and ln.split()[-1].startswith("/")})
        for p in paths:
            lib = ctypes.CDLL(p)
            for sym in ("scipy_openblas_get_num_threads64_", "scipy_openblas_get_num_threads",
                        "openblas_get_num_threads64_", "openblas_get_num_threads"):
                fn = getattr(lib, sym, None)
                if fn is not None:
                    fn.restype = ctypes.c_int
                    return {"library": os.path.basename(p), "threads": int(fn())}
    except OSError:
        pass
    return {"library": "unknown", "threads": None}


CPU_STAGES = 16


def cpu_pipeline(system):
    """The reference's RCCD.jl sweep on the host cores, as CPU_STAGES stages of real work."""
    from oracle.df_blocks import rccd_blocks_from_B
    from oracle.sampled import PipelinedSweep
    blocks = rccd_blocks_from_B(system.B, system.C, system.nocc)
    return PipelinedSweep(*blocks, system.eps, system.nocc, stages=CPU_STAGES)


def time_stages(sw, nsteps):
    """Run nsteps stages; the sweep time is the sum of the latest time of every stage when all
    were run (one whole sweep's arithmetic, measured), else the mean stage time x CPU_STAGES."""
    last, times = {}, []
    for _ in range(nsteps):
        k, dt = sw.step()
        last[k] = dt
        times.append(dt)
    if len(last) == sw.stages:
        return sum(last.values()), times, "measured"
    return statistics.mean(times) * sw.stages, times, "estimated"


def sample_text(n, how, stages_run, total_s):
    return (f"RCCD.jl-form sweep at nbf={n} (oracle restatement, FP64 numpy einsum/OpenBLAS, real "
            f"intermediates), cut into {CPU_STAGES} stages of real work per sweep (one stage per "
            f"step); {stages_run} stages timed ({total_s:.1f} s of CPU work); s/iter "
            + ("= sum of the latest time of each of the 16 stages (one whole sweep, measured)"
               if how == "measured" else "= mean stage time x 16 (fewer than 16 stages timed)"))


def run_reference(args):
    ws, rank, local, pg = dist_setup(args.gpus)
    if rank != 0:
        return
    from juesgpu.synthetic import make_named
    name, n, o, naux = SHAPE
    vir = n - o
    system = make_named(name)
    t_all = time.perf_counter()
    sw = cpu_pipeline(system)
    for _ in range(args.warmup):
        sw.step()
    v, times, how = time_stages(sw, args.steps)
    cores = os.cpu_count()
    blas = blas_threads()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s/iter", "n_gpus": 1,
            "steps": len(times), "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"rccd_{name.lower()}", "nbf": n, "nocc": o, "nvir": vir,
                       "naux": naux, "sweep": "RCCD.jl einsum form, FP64 numpy/OpenBLAS",
                       "step": f"one of {CPU_STAGES} stages of a sweep; value = s per whole sweep"},
            "sweep_s": v, "sweep_time": how, "stage_ms": [1e3 * t for t in times],
            "tflops_reference_flops": ccd_ref_flops(o, vir) / v / 1e12,
            "cpu_baseline": {"value": v, "unit": "s/iter", "cores": cores, "blas_threads": blas["threads"],
                             "blas": blas["library"], "kind": "port",
                             "sample": sample_text(n, how, len(times), sum(times))},
            "e2e": {"value": v, "unit": "s/iter", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t_all}
    print(json.dumps(line), flush=True)


def run_batch_measure(count, local, pg=None, precision="split"):
    """Batched MP2 energy + adjoint (one CUDA graph; in split precision each stage autotuned over
    the FP64 tile shapes and the grouped three-plane tcgen05 GEMM) against per-system launch
    loops of the single-system C-ABI call: in FP64 (the error reference) and in the batch's
    precision (the speed-up).  With several ranks the systems are sharded over them (independent
    units, no collective)."""
    from juesgpu import MollerPlesset
    from juesgpu.synthetic import batch_specs, make_system
    t0 = time.perf_counter()
    systems = []
    specs = batch_specs(count)
    for n, o, naux, sub in (pg.shard(specs) if pg is not None else specs):
        s = make_system(n, o, naux, seed=sub)
        systems.append((s.ao_eri(), np.asfortranarray(s.C), o, s.eps))
    gen_s = time.perf_counter() - t0
    loops = {}
    ref = None
    for prec in ("fp64", precision):
        t0 = time.perf_counter()
        res = [MollerPlesset.rmp2_adjoint(gao=g, C=C, nocc=o, eps=e, precision=prec, device=local)
               for g, C, o, e in systems]
        loops[prec] = time.perf_counter() - t0
        if prec == "fp64":
            ref = res
    # batched: first call plans, autotunes and captures the graph; then timed replays
    t0 = time.perf_counter()
    e_b, gbs, cbs, info = MollerPlesset.batch_rmp2(systems, adjoint=True, precision=precision, device=local)
    first_s = time.perf_counter() - t0
    reps = 3
    graph_ms = []
    t0 = time.perf_counter()
    for _ in range(reps):
        e_b, gbs, cbs, info = MollerPlesset.batch_rmp2(systems, adjoint=True, precision=precision, device=local)
        graph_ms.append(info.graph_ms)
    batch_s = (time.perf_counter() - t0) / reps
    if pg is not None:   # whole-job rates: every rank's share done
        loops = {k: pg.max(v) for k, v in loops.items()}
        first_s, batch_s = pg.max(first_s), pg.max(batch_s)
    err_e = max(abs(a - b[0]) for a, b in zip(e_b, ref))
    rel_g = max(float(np.linalg.norm(gb - b[1]) / np.linalg.norm(b[1])) for gb, b in zip(gbs, ref))
    rel_c = max(float(np.linalg.norm(cb - b[2]) / np.linalg.norm(b[2])) for cb, b in zip(cbs, ref))
    nbf = [g.shape[0] for g, _, _, _ in systems]
    return {"systems": count, "systems_this_rank": len(systems), "nbf_range": [min(nbf), max(nbf)],
            "precision": precision, "generate_s": gen_s,
            "loop_fp64_s": loops["fp64"], "loop_s": loops[precision],
            "loop_systems_per_s": count / loops[precision],
            "batch_first_call_s": first_s, "batch_s": batch_s, "batch_systems_per_s": count / batch_s,
            "speedup": loops[precision] / batch_s, "speedup_vs_fp64_loop": loops["fp64"] / batch_s,
            "graph_ms": statistics.median(graph_ms), "upload_ms": info.upload_ms,
            "download_ms": info.download_ms, "graph_nodes": info.graph_nodes,
            "stage_forms": [info.tile_shape[k] for k in range(info.nstages)],
            "stage_form_key": "0-3 FP64 tiles 64x64/32x64/64x32/32x32, 4 grouped three-plane tcgen05",
            "max_energy_error_eh": err_e, "max_gao_bar_rel_error": rel_g, "max_C_bar_rel_error": rel_c,
            "error_reference": "per-system FP64 single-system adjoint (jues_rmp2_adjoint)"}


def run_pT_measure(shape, local, precisions=("fp64", "split")):
    """(T) correction (jues_cc_pT) on a CCSD session's amplitudes after 8 DIIS sweeps."""
    from juesgpu.CoupledCluster import CCSession
    from juesgpu.synthetic import make_named
    import juesgpu
    w = make_named(shape).wfn()
    o, v = w.nalpha, w.Cav.shape[1]
    ses = CCSession(1, w, maxit=8, diis=True, r_conv=0.0, device=local, precision="split")
    ses.iterate(8)
    ctx = juesgpu.context(local)
    flops = 2.0 * v**3 * (v + o) * o * (o + 1) * (o + 2)
    out = {"workload": f"pT_{shape.lower()}", "nbf": w.Cao.shape[0], "nocc": o, "nvir": v,
           "flops_algorithmic": flops}
    for prec in precisions:
        ses.pT(prec)                       # warm-up (plans, packs, allocations)
        ctx.set_profiling(True)
        ctx.profile_reset()
        t0 = time.perf_counter()
        e = ses.pT(prec)
        wall = time.perf_counter() - t0
        w_ms, w_n = ctx.profile("pt_w")
        en_ms, _ = ctx.profile("pt_energy")
        pk_ms, _ = ctx.profile("pack_split")
        ctx.set_profiling(False)
        out[prec] = {"energy": e, "wall_s": wall, "gemm_ms": w_ms, "gemm_launches": w_n, "energy_ms": en_ms,
                     "pack_ms": pk_ms, "tflops_algorithmic_wall": flops / wall / 1e12}
    if "fp64" in out and "split" in out:
        out["split_minus_fp64_eh"] = out["split"]["energy"] - out["fp64"]["energy"]
        out["speedup"] = out["fp64"]["wall_s"] / out["split"]["wall_s"]
    ses.close()
    return out


def run_df_measure(shape, local, sweeps=5):
    """DF-RCCD (jues_df_rccd / jues_cc_create_df): the fitted factor of the synthetic system
    (its integrals are exactly B^T B) instead of the n^4 AO integrals.  Reports the session
    set-up (H2D of b, MO factors, the five blocks), split sweeps, and the whole C-ABI call with
    host buffers."""
    from juesgpu.CoupledCluster import CCSession, DFRCCD
    from juesgpu.synthetic import make_named
    from juesgpu.Wavefunction import wfn_from_rhf
    s = make_named(shape)
    b = np.asfortranarray(np.transpose(s.B, (1, 2, 0)))
    n = s.nbf
    w = wfn_from_rhf(s.C, s.eps, None, s.nocc)   # no n^4 array: the DF path reads C and eps
    t0 = time.perf_counter()
    ses = CCSession(0, w, pqP=b, guess="mp2", diis=True, r_conv=0.0, maxit=sweeps, device=local,
                    precision="split")
    setup = time.perf_counter() - t0
    ses.iterate(sweeps)
    lg = ses.log()
    ses.close()
    t0 = time.perf_counter()
    e = DFRCCD.do_df_rccd(w, b, maxit=sweeps, diis=True, precision="split", device=local)
    e2e = time.perf_counter() - t0
    return {"workload": f"df_rccd_{shape.lower()}_split", "nbf": n, "naux": s.naux, "setup_s": setup,
            "sweep_ms": sum(r[3] for r in lg) / len(lg), "e2e_s_per_iter": e2e / sweeps, "sweeps": sweeps,
            "h2d_bytes": int(b.nbytes), "energy": e}


def run_ccsd_measure(shape, gao, system, local, steps=3, fp64_steps=1):
    """RCCSD sweeps (jues_cc_create method 1) at the bench shape: split s/iter with its dominant
    GEMM's rate, one FP64 sweep on the same state, and the converged split energy at nbf=100
    against the FP64 golden."""
    import juesgpu
    from juesgpu.CoupledCluster import CCSession, RCCSD
    from juesgpu.synthetic import make_named
    ctx = juesgpu.context(local)
    o = system.nocc
    v = system.nbf - o
    ses = CCSession(1, gao=gao, Cocc=system.C[:, :o], Cvir=system.C[:, o:], eps=system.eps, device=local,
                    precision="split", diis=True, r_conv=0.0, refine=0, maxit=10**6)
    ses.iterate(2)
    ctx.set_profiling(True)
    ctx.profile_reset()
    m0 = len(ses.log())
    ses.iterate(steps)
    lg = ses.log()[m0:]
    s_iter = sum(r[3] for r in lg) / 1e3 / len(lg)
    prefixes = ("ccsd_pp_ladder", "ccsd_hh_ladder", "ccsd_x", "ccsd_ring", "ccsd_wj", "ccsd_wk", "ccsd_wabef",
                "ccsd_y", "ccsd_z", "ccsd_fae", "ccsd_fmi", "ccsd_t1", "pack_split", "t2_finalize")
    kms = {p: ctx.profile(p)[0] / steps for p in prefixes}
    pp_ms, pp_n = ctx.profile("ccsd_pp_ladder")
    pp_n -= ctx.profile("ccsd_pp_ladder.reduce")[1]
    ctx.set_profiling(False)
    fp64 = None
    if fp64_steps > 0:
        ses.set_precision("fp64")
        m1 = len(ses.log())
        ses.iterate(fp64_steps)
        fp64 = sum(r[3] for r in ses.log()[m1:]) / 1e3 / fp64_steps
    ses.close()
    pk, pk_kind = peaks()
    peak = pk.get("bf16_tflops_sustained", pk.get("bf16_tflops"))
    pp_exec = ladder_launch_flops(o, v)   # both ladders, K-stacked, one folded sign per launch
    pp_s = (pp_ms / pp_n / 1e3) if pp_n else None
    out = {"workload": f"rccsd_{shape.lower()}_split", "nbf": system.nbf, "nocc": o, "nvir": v,
           "s_per_iter": s_iter, "steps": len(lg), "fp64_s_per_iter": fp64,
           "speedup_vs_fp64": (fp64 / s_iter) if fp64 else None, "kernels_ms_per_step": kms,
           "dominant_kernel": "ccsd_pp_ladder", "dominant_launch_ms": 1e3 * pp_s if pp_s else None,
           "dominant_tflops_executed": pp_exec / pp_s / 1e12 if pp_s else None,
           "dominant_frac": (pp_exec / pp_s / 1e12 / peak) if pp_s else None,
           "peak_kind": f"{pk_kind} bf16 sustained"}
    # converged split RCCSD at nbf=100 against the FP64 oracle's energy
    ref = golden("S100").get("ccsd_diis", {}).get("energy")
    w100 = make_named("S100").wfn()
    t0 = time.perf_counter()
    e100, lg100 = RCCSD.do_rccsd(w100, maxit=60, diis=True, r_conv=0.0, e_conv=1e-8, precision="split",
                                 refine=0, device=local, return_log=True)
    out["converged_s100"] = {"energy": e100, "sweeps": len(lg100), "wall_s": time.perf_counter() - t0,
                             "error_eh": (e100 - ref) if ref is not None else None}
    return out


def run_gpu(args):
    ws, rank, local, pg = dist_setup(args.gpus)
    import juesgpu
    from juesgpu.CoupledCluster import CCSession, mRCCD
    from juesgpu.synthetic import make_named

    name, n, o, naux = SHAPE
    vir = n - o
    system = make_named(name, seed=rank)
    gao = system.ao_eri()
    Cocc, Cvir, eps = system.C[:, :o], system.C[:, o:], system.eps
    ctx = juesgpu.context(local)
    gold = golden(name) if rank == 0 else {}
    e_gold = gold.get("ccd_mp2guess_diis", {}).get("energy")

    # ---------------- resident sweeps (value): the default split setting ----------------
    t_setup = time.perf_counter()
    sess = CCSession(0, gao=gao, Cocc=Cocc, Cvir=Cvir, eps=eps, device=local, precision="split",
                     guess="mp2", diis=True, r_conv=0.0, refine=0, maxit=10**6)
    setup_s = time.perf_counter() - t_setup
    for _ in range(args.warmup):
        sess.iterate(1)
    ctx.set_profiling(True)
    ctx.profile_reset()
    n0 = len(sess.log())
    launches0 = ctx.launches()
    clk = ClockSampler(local)
    clk.start()
    clk.ready()
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sess.iterate(1)
    wall = time.perf_counter() - t0
    barrier(pg)
    clocks = clk.stop()
    launches = ctx.launches() - launches0
    log = sess.log()[n0:]
    dev_s = sum(r[3] for r in log) / 1e3
    pp_ms, pp_n = ctx.profile("ccd_pp_ladder")
    pp_n -= ctx.profile("ccd_pp_ladder.reduce")[1]      # split-K reductions are not GEMM launches
    ring_ms, ring_n = ctx.profile("ccd_ring")
    pack_ms, pack_n = ctx.profile("pack_split")
    gemm = {}   # the tcgen05 GEMM launches of the sweep by scope (split-K reductions taken out)
    for g in ccd_split_gemm_flops(o, vir):
        g_ms, g_n = ctx.profile(g)
        r_ms, r_n = ctx.profile(g + ".reduce")
        gemm[g] = (g_ms - r_ms, g_n - r_n)
    other_ms = {k: sum(ctx.profile(p)[0] for p in ps) / args.steps
                for k, ps in (("fae_fmi", ("fmi_trace", "fae_trace", "wp_fmi")),
                              ("x", ("ccd_x",)),
                              ("fold", ("pair_fold", "pair_unfold")),
                              ("wj_wk", ("ccd_wj", "ccd_wk")),
                              ("t2_finalize", ("t2_finalize",)),
                              ("t_tilde_axpby", ("t_tilde", "axpby")),
                              ("diis", ("diis_error", "lincomb")),
                              ("energy", ("dot",)))}
    ctx.set_profiling(False)
    dev_s = max_over_ranks(pg, dev_s)
    s_per_iter = dev_s / args.steps
    # ---------------- FP64 sweeps on the same state ----------------
    fp64 = None
    if args.fp64_steps > 0:
        sess.set_precision("fp64")
        m0 = len(sess.log())
        for _ in range(args.fp64_steps):
            sess.iterate(1)
        fp64 = sum(r[3] for r in sess.log()[m0:]) / 1e3 / args.fp64_steps
        sess.set_precision("split")
    sess.close()

    # ---------------- converged energies against the FP64 golden ----------------
    converged = None
    if args.check:
        converged = {}
        # the default split setting (three-plane integrals, split sweeps; split-only runs stop
        # when the energy changes by less than 0.1 uEh: their step norm and energy level off at
        # the split noise floor); the same with two closing FP64 sweeps; and the opt-in
        # two-plane integrals, which miss 1 uEh at this size
        for label, refine, tprec, rconv, econv in (("split", 0, None, 0.0, 1e-7),
                                                   ("split_refine2", 2, None, 1e-9, 0.0),
                                                   ("split2_integrals", 0, "split2", 0.0, 1e-7)):
            t0 = time.perf_counter()
            s2 = CCSession(0, gao=gao, Cocc=Cocc, Cvir=Cvir, eps=eps, device=local, precision="split",
                           guess="mp2", diis=True, r_conv=rconv, e_conv=econv, refine=refine, maxit=60,
                           transform_precision=tprec)
            t_setup = time.perf_counter() - t0
            s2.iterate(60)
            wall_c = time.perf_counter() - t0
            lg2 = s2.log()
            e_c = s2.energy()
            s2.close()
            converged[label] = {"energy": e_c, "sweeps": len(lg2), "fp64_sweeps": sum(1 for r in lg2 if r[4] == 0),
                                "setup_s": t_setup, "wall_s": wall_c,
                                "error_eh": (e_c - e_gold) if e_gold is not None else None}

    # ---------------- transform: <ij|ab> block + MP2 (library kernel events) ----------
    from juesgpu import MollerPlesset
    wt = system.wfn(ao_eri=gao)
    tr = {}
    for prec in ("fp64", "split", "split2"):
        ctx.set_profiling(True)
        ctx.profile_reset()
        e_mp2 = MollerPlesset.do_rmp2(wt, precision=prec, device=local)
        t_q, _ = ctx.profile("transform")
        t_p, _ = ctx.profile("pack_split")
        ctx.set_profiling(False)
        tr[prec] = {"ms": t_q + t_p, "mp2": e_mp2}
    mp2_golden = gold.get("mp2")
    transform = {"block": "<ij|ab> (ov|ov)", "fp64_ms": tr["fp64"]["ms"],
                 "split_ms": tr["split"]["ms"], "split_planes": 3,
                 "speedup": tr["fp64"]["ms"] / max(tr["split"]["ms"], 1e-9),
                 "mp2_fp64": tr["fp64"]["mp2"], "mp2_split": tr["split"]["mp2"],
                 "mp2_split_error_eh": tr["split"]["mp2"] - tr["fp64"]["mp2"],
                 "split2_ms": tr["split2"]["ms"], "mp2_split2": tr["split2"]["mp2"],
                 "mp2_split2_error_eh": tr["split2"]["mp2"] - tr["fp64"]["mp2"],
                 "mp2_fp64_vs_oracle_eh": (tr["fp64"]["mp2"] - mp2_golden) if mp2_golden else None}

    # ---------------- e2e: one converged C-ABI call with host buffers ----------------
    e2e = None
    if args.e2e_runs > 0:
        # the default split setting run to convergence (|dE| < 0.1 uEh) through mRCCD.do_rccd; the
        # host-to-device copy of the 12.8 GB AO integrals varies from run to run with the host's
        # page state, so the call is repeated and the median run is reported
        w = system.wfn(ao_eri=gao)
        runs = []
        for _ in range(args.e2e_runs):
            barrier(pg)
            ctx.set_profiling(True)
            ctx.profile_reset()
            t0 = time.perf_counter()
            e, lg = mRCCD.do_rccd(w, maxit=args.e2e_maxit, r_conv=0.0, e_conv=1e-7, guess="mp2",
                                  precision="split", refine=0, device=local, return_log=True)
            t_e2e = max_over_ranks(pg, time.perf_counter() - t0)
            e2e_kernels = {k: ctx.profile(k)[0] for k in ("", "transform", "pack_split", "ccd_")}
            e2e_host = {k: ctx.profile("host:" + k)[0] for k in ("h2d_ao_eri", "cc_create", "integral_blocks",
                                                                 "release_ao_eri")}
            # page-locking inside the AO-integral copy (part of h2d_ao_eri)
            e2e_host.update({"h2d_" + k: ctx.profile("h2d:" + k)[0] for k in ("register", "unregister")})
            e2e_kernels[""] -= ctx.profile("host:")[0] + ctx.profile("h2d:")[0]   # kernel events only
            e2e_host["register_failures"] = ctx.profile("host:register_failed")[1]
            ctx.set_profiling(False)
            runs.append((t_e2e, len(lg), e2e_kernels, e2e_host, e))
        runs.sort(key=lambda r: r[0])
        t_e2e, nsw, e2e_kernels, e2e_host, e_e2e = runs[len(runs) // 2]
        h2d = gao.nbytes + system.C.nbytes + eps.nbytes
        e2e = {"value": t_e2e / nsw, "unit": "s/iter", "h2d_bytes_per_step": int(h2d / nsw),
               "d2h_bytes_per_step": int(8 / nsw), "sweeps": nsw, "converged": nsw < args.e2e_maxit,
               "wall_s": t_e2e, "energy": e_e2e,
               "energy_error_eh": (e_e2e - e_gold) if e_gold is not None else None,
               "config": "precision=split (three-plane integrals, two-plane sweeps), MP2 guess, DIIS 6, "
                         "stop at |dE| < 1e-7 Eh",
               "wall_s_runs": [r[0] for r in runs], "h2d_ms_runs": [r[3]["h2d_ao_eri"] for r in runs],
               "kernel_ms": {("all" if k == "" else k): v for k, v in e2e_kernels.items()},
               "host_phase_ms": e2e_host,
               "includes": "H2D of AO ERIs, split transform of the 5 RCCD blocks, the sweeps to "
                           "convergence, energy read-back (median of the runs)"}

    ccsd = run_ccsd_measure(name, gao, system, local) if args.ccsd else None
    batch = run_batch_measure(args.batch, local, pg) if args.batch > 0 else None
    pT = run_pT_measure(args.pT_shape, local) if args.pT_shape != "none" else None
    df = run_df_measure(args.df_shape, local) if args.df_shape != "none" else None
    if rank != 0:
        return
    pk, pk_kind = peaks()
    # the dominant kernel: gett_tc_kernel<128,3,2,2>, every split GEMM launch of the sweep (three
    # products each); achieved = executed flops over all its launches / their summed duration
    peak = pk.get("bf16_tflops_sustained", pk.get("bf16_tflops"))
    gflops = ccd_split_gemm_flops(o, vir)
    g_s = sum(ms for ms, _ in gemm.values()) / 1e3
    g_n = sum(n_ for _, n_ in gemm.values())
    g_flops = 3 * sum(gflops.values()) * args.steps
    achieved = g_flops / g_s / 1e12 if g_s > 0 else None
    per_gemm = {g: {"ms_per_sweep": ms / args.steps, "launches_per_sweep": n_ / args.steps,
                    "tflops_executed": 3 * gflops[g] * args.steps / (ms / 1e3) / 1e12 if ms > 0 else None,
                    "frac": 3 * gflops[g] * args.steps / (ms / 1e3) / 1e12 / peak if ms > 0 else None}
                for g, (ms, n_) in gemm.items()}
    pp_flops_exec = ladder_launch_flops(o, vir)
    pp_avg_s = (pp_ms / pp_n / 1e3) if pp_n else None
    traffic = load_traffic().get(f"ccd_gemms_{name.lower()}")
    cpu = None
    if not args.skip_cpu and ws == 1:
        sw = cpu_pipeline(system)
        val, ct, how = time_stages(sw, args.cpu_steps)
        blas = blas_threads()
        cpu = {"value": val, "unit": "s/iter", "cores": os.cpu_count(), "blas_threads": blas["threads"],
               "blas": blas["library"], "kind": "port", "sample": sample_text(n, how, len(ct), sum(ct))}
    fp64_exec = ccd_exec_flops(o, vir)
    line = {
        "metric": METRIC, "value": s_per_iter, "unit": "s/iter", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * s_per_iter, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": SPLIT_DTYPE, "data": "synthetic",
        "config": {"workload": f"rccd_{name.lower()}_split", "nbf": n, "nocc": o, "nvir": vir, "naux": naux,
                   "parallelism": f"replicas{ws}", "l2": "inputs larger than L2 (packed folded vvvv 1.4 GB, T2 0.33 GB)",
                   "guess": "mp2", "diis": 6, "precision": "split (JUES_PREC_SPLIT)"},
        "replica_sweeps_per_s": ws / s_per_iter,
        "tflops_reference_flops": ccd_ref_flops(o, vir) / s_per_iter / 1e12,
        "tflops_executed_tensor": 3 * sum(ccd_split_gemm_flops(o, vir).values()) / s_per_iter / 1e12,
        "fp64_s_per_iter": fp64,
        "fp64_tflops_executed": (fp64_exec / fp64 / 1e12) if fp64 else None,
        "fp64_frac_of_spec": (fp64_exec / fp64 / 1e12 / FP64_SPEC_TFLOPS) if fp64 else None,
        "fp64_peak_note": f"GB300 FP64 {FP64_SPEC_TFLOPS} TFLOP/s, NVIDIA specification figure (not measured)",
        "speedup_vs_fp64": (fp64 / s_per_iter) if fp64 else None,
        "energy_fp64_golden": e_gold,
        "energy_error_eh": (converged or {}).get("split", {}).get("error_eh"),
        "converged_runs": converged,
        "transform": transform,
        "wall_s_timed": wall, "setup_s": setup_s,
        "kernels_ms_per_step": {"pp_ladder": pp_ms / args.steps, "ring": ring_ms / args.steps,
                                "pack_split": pack_ms / args.steps, **other_ms},
        "roofline": {"bound": "tensor",
                     "kernel": "gett_tc_kernel<128,3,2,2>, every tcgen05 split GEMM launch of the sweep (3 products): "
                               "X and the hole-hole + particle ladders folded over (i<=j), (a<=b), WmBeJ and the "
                               "rings K-stacked, WmBEj, the third ring",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": (achieved / peak) if achieved else None,
                     "peak_kind": f"{pk_kind} bf16 sustained",
                     "flops_per_launch": (g_flops / g_n) if g_n else None,
                     "launch_ms": (1e3 * g_s / g_n) if g_n else None, "launches_per_sweep": g_n / args.steps,
                     "per_gemm": per_gemm,
                     "ladder_launch": {"flops": pp_flops_exec, "ms": 1e3 * pp_avg_s if pp_avg_s else None,
                                       "frac": (pp_flops_exec / pp_avg_s / 1e12 / peak) if pp_avg_s else None},
                     "traffic": traffic},
        "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "gpu_launches": launches,
        "rccsd": ccsd, "batch": batch, "pT": pT, "df_rccd": df,
    }
    print(json.dumps(line), flush=True)


def run_gemm(args):
    """One jues_gemm call repeated (--warmup untimed, --steps timed with the library's events):
    a small standalone case for profiler captures of the operand pack and the GEMM kernel."""
    from juesgpu import _lib
    M, N, K = args.gemm
    rng = np.random.default_rng(0)
    A = np.asfortranarray(rng.standard_normal((M, K)))
    B = np.asfortranarray(rng.standard_normal((K, N)))
    ctx = _lib.context(0)
    for _ in range(args.warmup):
        _lib.gemm(A, B, precision=args.gemm_precision)
    ctx.set_profiling(True)
    ctx.profile_reset()
    for _ in range(args.steps):
        _lib.gemm(A, B, precision=args.gemm_precision)
    g_ms, g_n = ctx.profile("gemm")
    p_ms, p_n = ctx.profile("pack_split")
    ctx.set_profiling(False)
    products = {"split": 3, "split_bf16": 3, "split2": 3, "split3": 6, "fp64": 1}[args.gemm_precision]
    flops = 2.0 * M * N * K * products
    print(json.dumps({"gemm": [M, N, K], "precision": args.gemm_precision, "steps": args.steps,
                      "gemm_ms": g_ms / max(args.steps, 1), "pack_ms": p_ms / max(args.steps, 1),
                      "pack_launches": p_n, "tflops_executed": flops / (g_ms / args.steps * 1e-3) / 1e12
                      if g_ms > 0 else None}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=1)
    ap.add_argument("--e2e-runs", type=int, default=3, help="e2e calls; the median is reported")
    ap.add_argument("--e2e-maxit", type=int, default=60, help="sweep cap of the converged e2e call")
    ap.add_argument("--no-check", dest="check", action="store_false")
    ap.add_argument("--no-ccsd", dest="ccsd", action="store_false", help="skip the RCCSD sweep timing")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=CPU_STAGES, help="CPU baseline stages to time")
    ap.add_argument("--pT-shape", dest="pT_shape", default="S100", choices=["none"] + sorted(SHAPES),
                    help="(T) correction timing on this synthetic shape (FP64 and split)")
    ap.add_argument("--df-shape", dest="df_shape", default="S200", choices=["none"] + sorted(SHAPES),
                    help="DF-RCCD timing on this synthetic shape (split sweeps, set-up, C-ABI call)")
    ap.add_argument("--batch", type=int, default=512,
                    help="batched MP2 energy+adjoint form on this many systems (0 = skip)")
    ap.add_argument("--shape", default="S200", choices=sorted(SHAPES),
                    help="S200 is the benchmark; S100 is the small case used for profiler captures")
    ap.add_argument("--gemm", type=int, nargs=3, metavar=("M", "N", "K"), default=None,
                    help="instead: time one split GEMM C = A B (A M x K, B K x N, FP64 host arrays "
                         "through jues_gemm) -- the profiler case for the pack and GEMM kernels")
    ap.add_argument("--gemm-precision", default="split", choices=["split", "split_bf16", "split2", "split3", "fp64"])
    args = ap.parse_args()
    if args.gemm:
        run_gemm(args)
        return
    global SHAPE
    SHAPE = SHAPES[args.shape]
    if args.warmup < 3 and args.impl == "gb300":
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

"""Lanczos iterations per second on the 54^3 odd-l<=5 40x70 workload.

One step = one Lanczos iteration (H v with the sinc-DVR kinetic, rotor and
potential blocks, then the alpha/beta recurrence) over the packed odd-l block
of the 54^3 x (l<=5) basis of H2 in a 20-water SPC/E dodecahedral cage (seed
1), 40 Gauss-Legendre theta x 70 uniform phi nodes.  The inputs are synthetic
(generated cage, no external data).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Default arm: the mixed-precision GPU path timed with CUDA events on the
library's stream (value), the same metric end to end through the C ABI with
host buffers (e2e), the FP64 GPU path, the level accuracy of the mixed path
against the FP64 path at the same iteration count, the precision variants of
the same problem (iter/s and level errors of reduced kinetic slices, BF16
potential blocks and the CUDA-core kinetic), per-kernel times and the
roofline of the dominant kernel, and the CPU baseline (oracle restatement of
the reference's Hv and loop on the host cores, bounded sample).  Defaults:
10,000 timed iterations after 20, so that the timed region (about 1 s) spans
several 200 ms nvidia-smi clock samples; the working set (145 MB of potential
blocks) is larger than L2, so no flush is needed between iterations.
The launch shapes that the problem's size does not fix are picked by the
library's autotuner before the timed region.
--impl reference: only the CPU implementation, on the same workload: K
iterations after W warm-up ones (at most 3), on every host thread, bounded to
about a minute; rank 0 only.
--batched: only the batched workload (32 problems of uneven size, 3000
iterations each, inputs.batch_problems): total iterations/s of the grouped
batch, of one stream per problem and of one problem after another, and every
problem's levels against its FP64 run.
"""
import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "boundstate-lanczos_gb300")
ORACLE_LIB = os.path.join(REPO, "oracle", "_build", "liboracle.so")
METRIC = "Lanczos iter/s at 54³·l≤5 (mixed vs FP64 GPU) at ≤1e-3 cm⁻¹ level error"
UNIT = "iter/s"
KJ_TO_CM = 83.5935


def _load(name, path):
    import importlib.util
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def workload_files(tmp):
    inputs = _load("bsl_inputs", os.path.join(PKG, "inputs.py"))
    cfg = inputs.CONFIG_METRIC
    cage = os.path.join(tmp, "cage_seed%d.xyz" % cfg["cage_seed"])
    inputs.write_cage_xyz(cage, inputs.dodecahedral_cage(cfg["cage_seed"]))
    hv = os.path.join(tmp, "hv_input.txt")
    inputs.write_hv_input(hv, inputs.hv_fields(cfg["n"], cfg["x_max"], cfg["l_max"], cfg["theta_points"],
                                               cfg["phi_points"], cage, "metric_54_odd_l5", cfg["sym"]))
    return cfg, hv


def config_record(cfg, D=None, Df=None, precision="mixed"):
    rec = {"workload": "H2 in SPC/E dodecahedral cage (seed %d): %d^3 sinc-DVR grid over +-0.4 A, %s l<=%d, "
                       "%d theta x %d phi" % (cfg["cage_seed"], cfg["n"], cfg["sym"].lower(), cfg["l_max"],
                                              cfg["theta_points"], 2 * cfg["phi_points"]),
           "grid": cfg["n"], "l_max": cfg["l_max"], "symmetry": cfg["sym"], "theta_points": cfg["theta_points"],
           "phi_nodes": 2 * cfg["phi_points"], "precision": precision,
           "l2": "working set larger than L2 (potential blocks alone 145 MB FP32) - no flush needed"}
    if D is not None:
        rec["basis_packed"] = int(D)
        rec["basis_reference"] = int(Df)
    return rec


# --------------------------------------------------------------------------
# CPU baseline: the oracle restatement of the reference's Hv and Lanczos loop
# (serial kinetic, OpenMP potential blocks), on the same basis sizes with
# synthetic block values (the cost does not depend on the values).
# --------------------------------------------------------------------------
def cpu_baseline(cfg, budget_s=15.0, max_iters=30, warmup=1):
    """`warmup` untimed iterations (at least one, which also sizes the sample),
    then min(max_iters, budget_s / one iteration) timed iterations (at least 1)
    on every host thread, and one iteration on a single thread."""
    if not os.path.exists(ORACLE_LIB):
        subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "port"], check=True, capture_output=True)
    L = C.CDLL(ORACLE_LIB)
    L.orc_create_synthetic.restype = C.c_void_p
    L.orc_create_synthetic.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.c_char_p]
    L.orc_basis_size.restype = C.c_long
    L.orc_basis_size.argtypes = [C.c_void_p]
    P = C.POINTER(C.c_double)
    L.orc_lanczos.restype = C.c_double
    L.orc_lanczos.argtypes = [C.c_void_p, C.c_int, P, P, P, P, C.c_int]
    L.orc_destroy.argtypes = [C.c_void_p]
    cores = os.cpu_count() or 1
    h = C.c_void_p(L.orc_create_synthetic(cfg["n"], cfg["n"], cfg["n"], cfg["l_max"], cfg["x_max"], 2.01588,
                                          0.709648713, cfg["sym"].encode()))
    D = L.orc_basis_size(h)

    def run(n, threads=cores):
        a, b, b2 = np.zeros(n), np.zeros(n + 1), np.zeros(n + 1)
        return L.orc_lanczos(h, n, None, a.ctypes.data_as(P), b.ctypes.data_as(P), b2.ctypes.data_as(P), threads)

    t1 = run(1)
    for _ in range(max(0, warmup - 1)):
        run(1)
    n = int(max(1, min(max_iters, budget_s / max(t1, 1e-3))))
    t = run(n)
    t_one = run(1, threads=1)
    L.orc_destroy(h)
    return {"value": n / t, "unit": UNIT, "cores": cores, "kind": "port", "one_thread_value": 1.0 / t_one,
            "sample": "%d Lanczos iterations of the reference algorithm (oracle restatement: serial sinc-DVR "
                      "kinetic, OpenMP potential blocks, serial recurrence) on the %d-function reference basis "
                      "(%d^3 x (l_max+1)^2 with parity mask), %.1f s" % (n, D, cfg["n"], t),
            "seconds": t, "iterations": n, "basis_reference": D}


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples every 200 ms while the context is open; `summary`
    keeps the samples whose timestamps fall inside [start(), stop()]."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.t_start = self.t_stop = None

    def start(self):
        self.t_start = time.time()

    def stop(self):
        self.t_stop = time.time()

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def close(self):
        """Remove the sample file (after summary())."""
        try:
            os.unlink(self.path)
        except OSError:
            pass

    @staticmethod
    def _when(stamp):
        import datetime
        try:
            return datetime.datetime.strptime(stamp.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

    def summary(self):
        try:
            rows = [[c.strip() for c in l.split(",")] for l in open(self.path).read().strip().splitlines()
                    if l.strip()]
        except Exception:
            rows = []
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        inside = [r for r in rows if self.t_start is not None and self._when(r[0]) is not None
                  and self.t_start <= self._when(r[0]) <= self.t_stop]
        scope = "timed region" if inside else "whole sampler run (no sample fell inside the timed region)"
        rows = inside or rows
        num = lambda x: x.replace(".", "", 1).isdigit()
        sm = [float(r[2]) for r in rows if len(r) > 2 and num(r[2])]
        mx = [float(r[3]) for r in rows if len(r) > 3 and num(r[3])]
        pw = [float(r[4]) for r in rows if len(r) > 4 and num(r[4])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 6 + i and "Active" in r[6 + i]
                          and "Not" not in r[6 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_median": float(np.median(pw)) if pw else None, "reasons": reasons,
                "samples": len(rows), "scope": scope}


def measured_peak_hbm():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


# DRAM bytes (read + write) per launch of each mixed-path kernel in the running
# iteration: one-pass ncu capture with the L2 left as the previous kernel left it
# (the fused iteration of a run; the four-kernel iteration's potential stream
# and update from the earlier capture).
_TRAFFIC_SRC = "profiles/pipeline_traffic_warm_54cubed_odd_l5.md"
_FUSED_SRC = "profiles/fused_iteration_54cubed_odd_l5.md"
NCU_TRAFFIC = {"k_kin_xy_tc": (17.29e6, _FUSED_SRC),
               "k_kin_z_tc": (4.34e6, _FUSED_SRC),
               "k_vapply_light<NN>": (49.85e6, _FUSED_SRC),
               "k_vstream<NN,coefficients,update>": (68.43e6, _FUSED_SRC),
               "k_vstream<NN,coefficients>": (84.45e6, _TRAFFIC_SRC),
               "k_vstream<NN>": (200.97e6, _TRAFFIC_SRC),
               "k_update_stream": (9.05e6, _TRAFFIC_SRC)}


# potential values streamed per grid point in the spherical-harmonic form, by
# block size (csrc/bsl_gaunt.h: L <= 2 l_max of the block's parity)
GAUNT_ROWS = {21: 66, 15: 45, 10: 28}
VARIANT = {"gaunt": "V as FP32 spherical-harmonic coefficients (%d per point; blocks rebuilt per point)",
           "fp32": "V blocks, symmetric-packed FP32 (upper triangle, nn(nn+1)/2 per point)"}

# H v time of the compiled reference against the oracle port on the same input,
# 8 OpenMP threads, measured in the x86 container that has the reference tree
# (the reference is not on the GPU machine): the port is the faster of the two, so
# the CPU baseline understates the reference's time per iteration.
REFERENCE_VS_PORT_HV_MS = {"15^3 even l<=4": [3.6, 2.9], "27^3 odd l<=5": [37.4, 31.9],
                           "40^3 odd l<=5": [243.0, 166.0]}


def sync_ranks(dist):
    """Finish this rank's GPU work, then wait for every rank (replicas only:
    the ranks share nothing but this barrier and the timing maximum)."""
    import torch
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()


def max_over_ranks(x, dist):
    """The largest value of x over the ranks: the slowest replica's time."""
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, seconds, world):
    """Whole-job rate of world independent replicas (weak scaling): all the
    ranks' units over the slowest rank's time."""
    return world * units_per_rank / seconds


def stage_bytes(cfg, D, N, nn, mixed, rows=None, names=()):
    """Algorithmic bytes per launch of each stage of one Lanczos iteration;
    `rows` potential values streamed per grid point (default: the upper
    triangle of the block, nn (nn + 1) / 2); `names` the stage kernels
    (bsl_stage_times), which tell the layout of the iteration."""
    ntri = nn * (nn + 1) // 2 if rows is None else rows
    vb = ntri * N * (4 if mixed else 8)
    if any("k_vapply_light" in n for n in names):
        # graph-replayed iterations with the fused update: the block product
        # of the next v (FP32) is formed by the update and read by the apply
        return [2 * D * 8,          # kinetic x/y: read v, write u_kin
                3 * D * 8,          # kinetic z: read v, read+write u_kin
                4 * D * 8 + D * 4,  # light apply: v, u_kin, r (read+write), the product
                vb + 3 * D * 8 + D * 4]  # update + next product: coefficients, v, r (read+write), product write
    return [2 * D * 8,              # kinetic x/y: read v, write u_kin
            3 * D * 8,              # kinetic z: read v, read+write u_kin
            vb + 4 * D * 8,         # potential apply: blocks, v, u_kin, r (read+write)
            3 * (D + 1) * 8]        # r -= alpha v, beta^2: read v, r; write r (scales fold the swap)


def run_extra_launches(names):
    """Launches of a device-counted Lanczos run besides its iterations: the
    counter reset and the closing kernel of the deferred beta, and with the
    fused iteration the block product of the start vector."""
    return 3 if any("k_vapply_light" in n for n in names) else 2


def levels_of(bsl, a, b, b2, count):
    ev, _ = bsl.good_eigenvalues(a, b, b2, -1.0e3, 1.0e3)
    return ev


def stable_levels(bsl, a, b, b2, drop=200, tol=1e-9, unit=None):
    ev, _ = bsl.good_eigenvalues(a, b, b2, -1.0e3, 1.0e3, unit_roundoff=unit)
    n = len(a) - drop
    ev2, _ = bsl.good_eigenvalues(a[:n], b[:n + 1], b2[:n + 1], -1.0e3, 1.0e3, unit_roundoff=unit)
    return np.array([e for e in ev if len(ev2) and np.min(np.abs(ev2 - e)) <= tol])


# Precision variants of the metric problem: (name, potential blocks, kinetic
# engine, tensor-core slices); the Lanczos recurrence is double-float in all.
SWEEP = [("V fp32 spherical-harmonic coefficients, kinetic tensor-core 4 slices (exact, default)", "gaunt",
          "tensor", 4),
         ("V fp32 blocks, kinetic tensor-core 4 slices (exact)", "fp32", "tensor", 4),
         ("V fp32 coefficients, kinetic tensor-core 3 slices", "gaunt", "tensor", 3),
         ("V fp32 coefficients, kinetic tensor-core 2 slices (split 3-term)", "gaunt", "tensor", 2),
         ("V fp32 coefficients, kinetic tensor-core 1 slice (plain 9-bit)", "gaunt", "tensor", 1),
         ("V fp32 coefficients, kinetic CUDA-core fp32 head+tail", "gaunt", "simt", 4),
         ("V bf16 per-point scale, kinetic tensor-core 4 slices", "bf16", "tensor", 4),
         ("V bf16 per-point scale, kinetic tensor-core 2 slices", "bf16", "tensor", 2),
         ("V bf16 per-point scale, kinetic tensor-core 1 slice", "bf16", "tensor", 1)]


def level_errors(bsl, ref_levels, a, b, b2):
    """Per reference level, the distance (cm^-1) to the nearest level of a run,
    through the tail with the mixed path's tolerances and with the FP64 ones."""
    evm, _ = bsl.good_eigenvalues(a, b, b2, -1.0e3, 1.0e3, unit_roundoff=bsl.MIXED_UNIT_ROUNDOFF,
                                  rel_noise=bsl.MIXED_REL_NOISE)
    evr, _ = bsl.good_eigenvalues(a, b, b2, -1.0e3, 1.0e3)
    dev = np.array([np.min(np.abs(evm - e)) for e in ref_levels]) * KJ_TO_CM if len(evm) else np.full(
        len(ref_levels), np.inf)
    dev_r = np.array([np.min(np.abs(evr - e)) for e in ref_levels]) * KJ_TO_CM if len(evr) else np.full(
        len(ref_levels), np.inf)
    return dev, dev_r


def precision_sweep(bsl, h, ref_levels, n_it, fp64_rate, timed=2000):
    """One record per precision variant: iter/s (CUDA events, `timed`
    iterations after a warm-up run) and the level errors after n_it iterations
    against the FP64 levels at the same iteration count."""
    recs = [{"variant": "V fp64, kinetic fp64 (the FP64 path)", "iter_s": fp64_rate, "max_abs_dE_cm-1": 0.0,
             "levels_within_1e-3_cm-1": len(ref_levels)}]
    h.set_precision("mixed")
    default_format = h.potential_format()
    for name, vfmt, engine, slices in SWEEP:
        h.set_potential_format(vfmt)
        h.set_kinetic_engine(engine)
        h.set_kinetic_slices(slices)
        h.lanczos(64)
        h.lanczos(timed)
        rate = 1000.0 / h.last_ms_per_iter()
        a, b, b2 = h.lanczos(n_it, start="normal", seed=0)
        dev, dev_r = level_errors(bsl, ref_levels, a, b, b2)
        recs.append({"variant": name, "iter_s": rate, "max_abs_dE_cm-1": float(dev.max()),
                     "max_abs_dE_cm-1_lowest20": float(dev[:20].max()),
                     "levels_within_1e-3_cm-1": int(np.sum(dev <= 1e-3)),
                     "max_abs_dE_cm-1_fp64_tail_tolerance": float(dev_r.max()),
                     "levels_within_1e-3_cm-1_fp64_tail_tolerance": int(np.sum(dev_r <= 1e-3))})
    h.set_potential_format(default_format)
    h.set_kinetic_slices(4)
    h.set_kinetic_engine("tensor")
    return recs


def batched_workload(bsl, tmp, device, fp64_check=True, nlev=10):
    """The batched workload (inputs.batch_problems: 32 uneven problems, 3000
    iterations each): total Lanczos iterations per second of all the problems
    through bsl_lanczos_run_batch (device time of the whole batch, the
    iteration graphs cached by a warm-up batch), against the same problems run
    one after another; and, per problem, the lowest `nlev` converged FP64
    levels against the batched mixed run's levels at the same iteration
    count."""
    inputs = _load("bsl_inputs", os.path.join(PKG, "inputs.py"))
    probs = inputs.batch_problems()
    hs = []
    t0 = time.perf_counter()
    for k, pr in enumerate(probs):
        cage = os.path.join(tmp, "batch_cage%d.xyz" % pr["cage_seed"])
        if not os.path.exists(cage):
            inputs.write_cage_xyz(cage, inputs.dodecahedral_cage(pr["cage_seed"], pr["radius"]))
        hv = os.path.join(tmp, "batch_hv%d.txt" % k)
        inputs.write_hv_input(hv, inputs.hv_fields(pr["n"], pr["x_max"], pr["l_max"], pr["theta_points"],
                                                   pr["phi_points"], cage, "batch%d" % k, pr["sym"]))
        hs.append(bsl.Hamiltonian(hv, "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE", precision="mixed",
                                  device=device))
    prep_s = time.perf_counter() - t0
    niter = probs[0]["niter"]
    total = len(probs) * niter
    tune = bsl.autotune(hs, 64)  # launch shapes of the grouped batch
    bsl.lanczos_batch(hs, 64, start="normal", seed=0)  # warm-up
    runs = bsl.lanczos_batch(hs, niter, start="normal", seed=0)
    batch_ms = hs[0].last_ms_per_iter() * niter
    bsl.lanczos_batch(hs, 64, start="normal", seed=0, grouped=False)  # warm-up: per-problem graphs cached
    bsl.lanczos_batch(hs, niter, start="normal", seed=0, grouped=False)
    streams_ms = hs[0].last_ms_per_iter() * niter
    sep_ms = 0.0
    for h in hs:
        h.lanczos(niter, start="normal", seed=0)
        sep_ms += h.last_ms_per_iter() * niter
    rec = {"problems": len(probs), "iterations_each": niter,
           "coefficients_total": int(sum(h.packed_size for h in hs)),
           "edges": [pr["n"] for pr in probs], "blocks": [h.nn for h in hs],
           "batched_iter_s": total / (batch_ms * 1e-3), "batched_ms": batch_ms,
           "path": "bsl_lanczos_run_batch: four grouped launches per iteration of all the problems "
                   "(each CTA on one problem), 32-iteration graph",
           "streams_iter_s": total / (streams_ms * 1e-3), "streams_ms": streams_ms,
           "streams_path": "bsl_lanczos_run_batch_streams: one stream per problem, 32-iteration graphs "
                           "interleaved",
           "sequential_iter_s": total / (sep_ms * 1e-3), "sequential_ms": sep_ms,
           "prep_seconds": prep_s,
           "launch_shapes": {"potential_stream_ctas_per_sm": tune[0], "update_ctas_per_sm": tune[1],
                             "by": "bsl_autotune"}}
    if fp64_check:
        worst, within, cnt = 0.0, 0, 0
        for h, (am, bm, bm2) in zip(hs, runs):
            h.set_precision("fp64")
            a, b, b2 = h.lanczos(niter, start="normal", seed=0)
            ref = np.sort(stable_levels(bsl, a, b, b2))[:nlev]
            dev, _ = level_errors(bsl, ref, am, bm, bm2)
            worst = max(worst, float(dev.max()))
            within += int(np.sum(dev <= 1e-3))
            cnt += len(ref)
        rec.update({"levels_compared": cnt, "levels_within_1e-3_cm-1": within, "max_abs_dE_cm-1": worst})
    for h in hs:
        h.close()
    return rec


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--accuracy-iters", type=int, default=10000)
    ap.add_argument("--fp64-steps", type=int, default=200)
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--profile-iters", type=int, default=0,
                    help="prep plus this many iterations only (for profiler captures)")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--dump-lanczos", default="",
                    help="save the alpha/beta histories of the accuracy runs to this .npz file")
    ap.add_argument("--batched", action="store_true",
                    help="only the batched workload (32 uneven problems, 3000 iterations each)")
    ap.add_argument("--sweep", type=int, default=1,
                    help="1: add the precision variants of the metric problem (iter/s and level errors against "
                         "the FP64 levels at --accuracy-iters iterations) to the line; 0: skip")
    ap.add_argument("--kinetic", default="auto", choices=["auto", "simt", "tensor"],
                    help="kinetic engine of the mixed path (auto: tensor cores where the grid allows)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    tmp = tempfile.mkdtemp()
    cfg, hv_path = workload_files(tmp)

    if args.impl == "reference":
        if rank != 0:
            return
        # a step is one Lanczos iteration of the reference algorithm; K steps
        # after W warm-up ones, bounded to about a minute of host time
        warm = max(1, min(args.warmup, 3))
        cb = cpu_baseline(cfg, budget_s=60.0, max_iters=max(1, args.steps), warmup=warm)
        line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": cb["iterations"],
                "warmup": warm, "ms_per_step": 1000.0 / cb["value"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (generated cage; block values synthetic)",
                "config": config_record(cfg, precision="fp64"), "impl": "reference",
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "one_thread_value")},
                "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if cb["iterations"] != args.steps:
            line["requested_steps"] = args.steps  # bounded to about a minute of host time
        print(json.dumps(line))
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    bsl = _load("boundstate_lanczos_gb300", os.path.join(PKG, "__init__.py"))
    if args.batched:
        rec = batched_workload(bsl, tmp, local)
        print(json.dumps(dict(record="batched workload: 16 cages x {ortho odd l<=5, para even l<=4}, edges "
                                     "from {27, 33, 41}, 24 theta x 48 phi, 3000 iterations each", **rec)))
        return
    t0 = time.perf_counter()
    h = bsl.Hamiltonian(hv_path, "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE", precision=args.precision, device=local)
    prep_s = time.perf_counter() - t0
    if args.kinetic != "auto":
        h.set_kinetic_engine(args.kinetic)
    kinetic_engine = h.kinetic_engine()
    gaunt_resid = h.gaunt_residual()
    D, Df, nn = h.packed_size, h.basis_size, h.nn
    N = D // nn
    if args.profile_iters:
        # short run for profilers: prep, then the given number of iterations only
        h.lanczos(args.profile_iters)
        torch.cuda.synchronize()
        print(json.dumps({"profile_iters": args.profile_iters, "ms_per_iter": h.last_ms_per_iter(),
                          "precision": args.precision, "kinetic": h.kinetic_engine()}))
        h.close()
        return

    def barrier():
        sync_ranks(dist)

    # ---- device-resident mixed path (value) ----
    # launch shapes picked by the library's autotuner (outside the timed region)
    tune = bsl.autotune([h], 100)
    h.lanczos(max(3, args.warmup))
    barrier()
    with ClockSampler(local) as clk:
        clk.start()
        t0 = time.perf_counter()
        h.lanczos(args.steps)
        barrier()
        wall = time.perf_counter() - t0
        clk.stop()
        time.sleep(0.25)  # the sample that covers the end of the region
    ms_event = h.last_ms_per_iter()
    ms_step = max_over_ranks(ms_event, dist)
    value = replica_rate(1000.0, ms_step, world)

    # ---- per-kernel times (CUDA events around each launch on the library stream) ----
    stage_ms = np.zeros(5)
    names = (C.c_char_p * 5)()
    bsl.lib().bsl_stage_times.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_void_p]
    rc = bsl.lib().bsl_stage_times(h.handle, 200, stage_ms.ctypes.data_as(C.POINTER(C.c_double)), names)
    nst = bsl.lib().bsl_launches_per_iteration(h.handle)
    stage_names = [names[i].decode() for i in range(nst)] if rc == 0 else []
    stage_ms = stage_ms[:nst]
    vfmt = h.potential_format()
    rows = {"gaunt": GAUNT_ROWS.get(nn), "fp32": None}.get(vfmt)
    sb = stage_bytes(cfg, D, N, nn, True, rows, stage_names)[:nst]
    peak, peak_src = measured_peak_hbm()
    dom = int(np.argmax(stage_ms))
    achieved = sb[dom] / (stage_ms[dom] * 1e-3) / 1e9
    it_bytes = sum(sb)

    # ---- end to end through the C ABI with host buffers (pinned) ----
    vec = torch.empty(Df, dtype=torch.float64, pin_memory=True).numpy()
    rvec = torch.empty(Df, dtype=torch.float64, pin_memory=True).numpy()
    vec[:] = 1.0 / math.sqrt(Df)
    rvec[:] = 0.0
    for _ in range(3):
        h.step_host(vec, rvec)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        h.step_host(vec, rvec)
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e_value = replica_rate(args.e2e_steps, e2e_s, world)
    # the transfer floor of that path: the same bytes between pinned host memory
    # and the device through torch, each direction on its own
    dv = torch.empty(Df, dtype=torch.float64, device="cuda")
    tv, tr = torch.from_numpy(vec), torch.from_numpy(rvec)
    ev0, ev1, ev2 = torch.cuda.Event(True), torch.cuda.Event(True), torch.cuda.Event(True)
    torch.cuda.synchronize()
    ev0.record()
    for _ in range(5):
        dv.copy_(tv, non_blocking=True)
        dv.copy_(tr, non_blocking=True)
    ev1.record()
    for _ in range(5):
        tv.copy_(dv, non_blocking=True)
        tr.copy_(dv, non_blocking=True)
    ev2.record()
    torch.cuda.synchronize()
    h2d_ms, d2h_ms = ev0.elapsed_time(ev1) / 5, ev1.elapsed_time(ev2) / 5

    # ---- FP64 GPU path ----
    h.set_precision("fp64")
    h.lanczos(3)
    h.lanczos(args.fp64_steps)
    fp64_ms = h.last_ms_per_iter()
    fp64_stage = np.zeros(5)
    bsl.lib().bsl_launches_per_iteration.argtypes = [C.c_void_p]
    bsl.lib().bsl_stage_times(h.handle, 20, fp64_stage.ctypes.data_as(C.POINTER(C.c_double)), None)

    # ---- level accuracy: mixed vs FP64 at the same iteration count ----
    acc = {}
    sweep = None
    if args.accuracy_iters > 0 and rank == 0:
        n_it = args.accuracy_iters
        a64, b64, b264 = h.lanczos(n_it, start="normal", seed=0)
        h.set_precision("mixed")
        am, bm, bm2 = h.lanczos(n_it, start="normal", seed=0)
        if args.dump_lanczos:
            np.savez(args.dump_lanczos, a64=a64, b64=b64, b264=b264, am=am, bm=bm, bm2=bm2)
        ref_levels = np.sort(stable_levels(bsl, a64, b64, b264))[:cfg["levels"]]
        # the mixed levels through the tail with the mixed path's tolerances
        # (bsl_good_eigenvalues_noise); the reference tail's FP64 tolerance is reported beside
        dev, dev_r = level_errors(bsl, ref_levels, am, bm, bm2)
        worst = int(np.argmax(dev)) if len(dev) else -1
        acc = {"iterations": n_it, "levels_compared": int(len(ref_levels)),
               "max_abs_dE_cm-1": float(dev.max()) if len(dev) else None,
               "max_abs_dE_cm-1_lowest20": float(dev[:20].max()) if len(dev) else None,
               "levels_within_1e-3_cm-1": int(np.sum(dev <= 1e-3)),
               "median_abs_dE_cm-1": float(np.median(dev)) if len(dev) else None,
               "worst_level_kJ_mol": float(ref_levels[worst]) if worst >= 0 else None,
               "dE_cm-1_per_level": [float("%.3g" % x) for x in dev],
               "tail_unit_roundoff_mixed": bsl.MIXED_UNIT_ROUNDOFF, "tail_rel_noise_mixed": bsl.MIXED_REL_NOISE,
               "levels_within_1e-3_cm-1_fp64_tail_tolerance": int(np.sum(dev_r <= 1e-3)),
               "min_level_gap_cm-1": float(np.min(np.diff(ref_levels)) * KJ_TO_CM) if len(ref_levels) > 1 else None,
               "lowest_levels_kJ_mol": [float(x) for x in ref_levels[:5]], "start": "normal seed 0"}
        # one H v at full size, mixed against FP64
        vr = np.random.default_rng(3).standard_normal(Df)
        u64 = np.zeros(Df)
        um = np.zeros(Df)
        h.set_precision("fp64")
        h.hv(vr, u64)
        h.set_precision("mixed")
        h.hv(vr, um)
        acc["hv_rel_err_mixed_vs_fp64"] = float(np.max(np.abs(um - u64)) / np.max(np.abs(u64)))
        if args.sweep:
            sweep = precision_sweep(bsl, h, ref_levels, n_it, 1000.0 / fp64_ms)
    h.close()

    cb = cpu_baseline(cfg, budget_s=args.cpu_budget) if rank == 0 else None
    clocks = clk.summary()
    clk.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (generated SPC/E cage, seed 1)",
        "config": dict(config_record(cfg, D, Df), kinetic_engine=kinetic_engine),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * Df * 8, "d2h_bytes_per_step": 2 * Df * 8,
                "ms_per_step": 1000.0 / e2e_value * world, "h2d_ms_per_step": h2d_ms, "d2h_ms_per_step": d2h_ms,
                "path": "bsl_lanczos_step_host: reference loop body with host (pinned) vec/rvec in the reference "
                        "layout, H2D + Hv + recurrence + D2H per step"},
        "roofline": {"bound": "hbm", "kernel": stage_names[dom] if stage_names else None,
                     "variant": (VARIANT[vfmt] % GAUNT_ROWS[nn]) if vfmt == "gaunt" else VARIANT.get(vfmt, vfmt),
                     "gaunt_residual_kJ_mol": gaunt_resid,
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (NCU_TRAFFIC[stage_names[dom]][0]
                                 if stage_names and stage_names[dom] in NCU_TRAFFIC else None),
                     "traffic_source": (NCU_TRAFFIC[stage_names[dom]][1]
                                        if stage_names and stage_names[dom] in NCU_TRAFFIC else None),
                     "peak_source": peak_src + " (of measured)",
                     "algorithmic_bytes_per_launch": sb[dom], "ms_per_launch": float(stage_ms[dom]),
                     "dram_frac": (NCU_TRAFFIC[stage_names[dom]][0] / (stage_ms[dom] * 1e-3) / 1e9 / peak
                                   if stage_names and stage_names[dom] in NCU_TRAFFIC else None)},
        "iteration_roofline": {"bytes_per_iteration": it_bytes,
                               "achieved_GBs": it_bytes / (ms_step * 1e-3) / 1e9 / world,
                               "frac": it_bytes / (ms_step * 1e-3) / 1e9 / world / peak},
        "stages_ms": dict(zip(stage_names, [float(x) for x in stage_ms])),
        "fp64": {"value": 1000.0 / fp64_ms, "unit": UNIT, "ms_per_step": fp64_ms,
                 "stages_ms": [float(x) for x in fp64_stage[:nst]], "speedup_mixed_vs_fp64": fp64_ms / (ms_step)},
        "accuracy": acc,
        "precision_sweep": sweep,
        "cpu_baseline": dict({k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "one_thread_value")},
                             reference_vs_port_hv_ms=REFERENCE_VS_PORT_HV_MS,
                             reference_vs_port_note="compiled reference vs this port, H v ms, 8 threads, x86 "
                                                    "build container; the port is faster, so the baseline is "
                                                    "conservative"),
        "clocks": clocks, "gpu_launches": nst * args.steps + run_extra_launches(stage_names), "prep_seconds": prep_s,
        "launch_shapes": {"potential_stream_ctas_per_sm": tune[0], "update_ctas_per_sm": tune[1],
                          "autotune_ms_per_iter": tune[2], "by": "bsl_autotune"},
        "wall_ms_per_step": 1000.0 * wall / args.steps,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()

#!/usr/bin/env python
"""Throughput of the COORDINATION hot path on one GB300 (or N, one process each).

Workload (the 262,144-atom configuration the headline target is quoted on):
  262,144 atoms on a jittered 64^3 simple-cubic lattice (sigma 0.03 nm) filling
  a periodic 19.87 nm cube; GROUPA = all atoms (single list);
  SWITCH={RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.6}; NLIST NL_CUTOFF=0.8
  NL_STRIDE=10; 16 independent walkers (separately seeded) per GPU, batched in
  one launch per kernel; mixed precision (FP32 pair math, FP64 compensated
  sums).  A step is CV + derivatives + virial for all walkers, followed by the
  backward pass of a 500-hill metadynamics-style bias when it is available.
  Neighbour lists are rebuilt on steps that are multiples of NL_STRIDE, so
  rebuilds are amortised exactly as in an MD run; between rebuilds the walkers
  move by Gaussian steps of 0.002 nm per coordinate (step k uses frame k % 10
  of a 10-frame trajectory that starts at the lattice frame).

  value  = pair-evaluations (neighbour-list entries processed, summed over
           walkers) per second, inputs resident in HBM, CUDA events around the
           timed steps on the library's stream.  Working set per step (FP64
           positions 100 MB + neighbour lists ~0.7 GB) exceeds the 129 MB L2.
  e2e    = the same metric through the C ABI's host-array call
           (coord_forward_batch: all walkers' pinned host arrays in one call,
           positions in and s/derivatives/virial out inside the timed
           region, lists rebuilt every 10th step, timed after one untimed
           stride in which the context tunes its passes); e2e.per_walker_call
           is the plugin's call (coord_forward, one context and one call per
           walker, each walker's position array rewritten in place between
           steps as an MD engine does).

  --impl reference : the reference's algorithm on the host cores (the C
  restatement in oracle/, pinned in the tests against the reference's own code
  built as oracle/_ref), OpenMP over all threads, one walker per step, each
  step charged its pair loop + 1/10 of the serial cell-list build.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "CV+force µs/step & pair-evals/s, mixed+batched vs FP64 GPU at ≤1e-6 rel err"
N_ATOMS = 262144
BOX = 19.87
SPEC = "RATIONAL R_0=0.32 NN=6 MM=12 D_MAX=0.6"
LINE = "GROUPA=1-%d SWITCH={%s} NLIST NL_CUTOFF=0.8 NL_STRIDE=10"
MOTION_SIGMA = 0.002  # nm per coordinate per step: the walkers move as in an MD run between rebuilds
ALG_FLOPS_PER_PAIR = 57  # FMA = 2: delta 3, min-image 9, r^2 5, switch+dfunc 12, chain 4, dd 3, derivs 6, virial 18, s 1


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--walkers", type=int, default=16)
    ap.add_argument("--atoms", type=int, default=N_ATOMS)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true", help="small sizes (for profiling captures)")
    ap.add_argument("--c2-steps", type=int, default=3,
                    help="timed graph replays of the batched 256-action workload (0: skip it)")
    ap.add_argument("--workload", default="c4", choices=["c4", "c3", "c2", "c1", "c0"],
                    help="c3 / c2 / c1 / c0: only that workload, as its own line")
    return ap.parse_args()


def e2e_pairs(n_first: int, n_last: int, steps: int) -> int:
    """Pair-evaluations of steps 1..steps after a build at step 0: the lists
    rebuilt at step 10 (NL_STRIDE) serve the steps from 10 on."""
    later = max(0, steps - 9)
    return n_first * (steps - later) + n_last * later


E2E_WINDOWS = 3  # timed windows of the end-to-end calls (the median is reported)

HOST_PATH_TEXT = {
    "chunked": "page-locked arrays on the copy engines, the walkers in four chunks beside the kernels of the "
               "other chunks",
    "direct": "kernels reading and writing the caller's arrays in place through the host page tables",
    "staged": "staged through the context's pinned buffers",
}


def host_path_note(counts):
    """How the timed host-array calls moved the caller's arrays, as the library reported each call
    (coord_host_path): every path with its number of calls."""
    total = sum(counts.values())
    return "; ".join("%s: %d of %d calls" % (HOST_PATH_TEXT.get(k, str(k)), v, total)
                     for k, v in sorted(counts.items(), key=lambda kv: -kv[1]))


def measure_e2e(make_ctx, hp, hs, hd, hv, box, W, n, steps, addr):
    """The end-to-end figures through the host-array C ABI: the batched call
    (coord_forward_batch) over page-locked frames hp[T][W][n][3] with results
    in hs, hd, hv, and the plugin's call (coord_forward) per walker on
    pageable arrays.  Returns (batched value, its windows, its host paths,
    per-walker value, its windows, its host paths); values in pair-evals/s."""
    # all walkers in one call, page-locked host arrays
    T = hp.shape[0]
    cb = make_ctx()
    hb = np.ascontiguousarray(np.stack([box.reshape(9)] * W))
    A = (addr(hb), addr(hs), addr(hd), addr(hv))
    # steps 0..10 untimed (the context's first calls tune its passes), then the timed steps 11..
    for k in range(0, 11):
        cb.forward_host_batch(W, addr(hp[k % T]), A[0], k, 0, A[1], A[2], A[3])
    # three windows of `steps` steps (11.., then the next two), each ending on a rebuild step; the
    # median window is reported, every window listed, and how each timed call moved the arrays counted
    e2e_windows, batch_paths, k0 = [], {}, 11
    for _ in range(E2E_WINDOWS):
        n_first = sum(cb.nl_size(w) for w in range(W))  # the lists of the window's first steps
        te_b = 0.0
        for k in range(k0, k0 + steps):
            t0 = time.perf_counter()
            cb.forward_host_batch(W, addr(hp[k % T]), A[0], k, 0, A[1], A[2], A[3])
            te_b += time.perf_counter() - t0
            batch_paths[cb.host_path()] = batch_paths.get(cb.host_path(), 0) + 1
        e2e_windows.append(e2e_pairs(n_first, sum(cb.nl_size(w) for w in range(W)), steps) / te_b)
        k0 += steps
    assert np.all(np.isfinite(hs)) and np.all(hs > 0)
    e2e_v = float(np.median(e2e_windows))
    cb.close()
    ctxs = [make_ctx() for _ in range(W)]
    # one pageable position array per walker, which the MD engine rewrites in place every step (outside
    # the timed calls, as the integrator's update is not PLUMED's); force and virial arrays reused from
    # step to step.  The call is the C ABI's coord_forward with the arrays' addresses, as the PLUMED
    # plugin makes it.  (A fresh array per step, never an MD engine's pattern, runs about 1.5x slower on
    # the direct host path: each first GPU touch of host pages costs address translations.)
    host_pos = [np.array(hp[0, w]) for w in range(W)]
    outs = [(np.zeros((n, 3)), np.zeros(9), np.zeros(1)) for _ in range(W)]
    hbox = np.ascontiguousarray(box.reshape(9))
    ptrs = [(addr(outs[w][2]), addr(outs[w][0]), addr(outs[w][1])) for w in range(W)]
    pptr = [addr(host_pos[w]) for w in range(W)]
    for w in range(W):
        ctxs[w].forward_host(pptr[w], addr(hbox), 0, 0, ptrs[w][0], ptrs[w][1], ptrs[w][2])
    # one stride untimed (each context tunes its passes on its first calls), then the timed steps
    for k in range(1, 11):
        for w in range(W):
            np.copyto(host_pos[w], hp[k % T, w])
            ctxs[w].forward_host(pptr[w], addr(hbox), k, 0, ptrs[w][0], ptrs[w][1], ptrs[w][2])
    walker_windows, walker_paths, k0 = [], {}, 11
    for _ in range(E2E_WINDOWS):
        n_first = sum(ctxs[w].nl_size() for w in range(W))
        te = 0.0
        for k in range(k0, k0 + steps):
            for w in range(W):
                np.copyto(host_pos[w], hp[k % T, w])  # the MD engine's position update
            t0 = time.perf_counter()
            for w in range(W):
                ctxs[w].forward_host(pptr[w], addr(hbox), k, 0, ptrs[w][0], ptrs[w][1], ptrs[w][2])
            te += time.perf_counter() - t0
            for w in range(W):
                walker_paths[ctxs[w].host_path()] = walker_paths.get(ctxs[w].host_path(), 0) + 1
        walker_windows.append(e2e_pairs(n_first, sum(ctxs[w].nl_size() for w in range(W)),
                                        steps) / te)
        k0 += steps
    # the results landed in the caller's arrays
    assert all(np.isfinite(outs[w][2][0]) and outs[w][2][0] > 0 for w in range(W))
    e2e_walker = float(np.median(walker_windows))
    for x in ctxs:
        x.close()
    return e2e_v, e2e_windows, batch_paths, e2e_walker, walker_windows, walker_paths


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi samples during the timed region (median SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        # the raw samples (summarised in the JSON line); COORD_BENCH_CLOCKS_DIR keeps them elsewhere
        out_dir = os.environ.get("COORD_BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, "clocks_bench_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def _one_shot(self):
        """One query at the end of a timed region too short for the loop's
        first sample (lines in the loop's format; none if it fails)."""
        try:
            r = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=10)
            return r.stdout.splitlines()
        except Exception:
            return []

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        extra = []
        try:
            self.f.flush()
            if not any(len(x.split(",")) >= 9 for x in open(self.path)):
                extra = self._one_shot()
        except Exception:
            extra = []
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in list(open(self.path)) + extra:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
            if extra:
                out["one_shot_at_end"] = True
        return out


PROFILE_EVAL = os.path.join(ROOT, "profiles", "k_eval_nl32_110592atoms_16walkers.md")


def eval_traffic(bytes_alg):
    """DRAM bytes (read + write) per pair-kernel launch from the committed ncu summary of a smaller launch, scaled
    by the ratio of algorithmic bytes; None without the summary."""
    got = {}
    try:
        for line in open(PROFILE_EVAL):
            for key in ("traffic_bytes_per_launch", "alg_bytes_per_launch"):
                if line.startswith(key + ":"):
                    got[key] = float(line.split(":", 1)[1])
    except OSError:
        return None
    if len(got) < 2:
        return None
    return got["traffic_bytes_per_launch"] * bytes_alg / got["alg_bytes_per_launch"]


def rank_walkers(rank, walkers_per_rank):
    """Walker seeds a rank owns: disjoint blocks, so N ranks run N x the walkers with no exchange
    (weak scaling)."""
    return list(range(rank * walkers_per_rank, (rank + 1) * walkers_per_rank))


def reduce_over_ranks(x, op="max", device=None):
    """x reduced over the ranks of the default process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return x
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return t.item()


def make_walkers(n_walkers, n_atoms, first):
    """Jittered simple-cubic lattices at the 262,144-atom system's spacing (19.87 / 64 nm) filling a cube
    of m = n_atoms^(1/3) sites per side (n_atoms a cube: smaller systems for profiling captures)."""
    from plumed2_gb300.frames import sc_sites
    sites = sc_sites(n_atoms)
    m = round(n_atoms ** (1 / 3))
    if m ** 3 != n_atoms:
        raise ValueError("the atom count must be a cube, not %d" % n_atoms)
    a = BOX / round(N_ATOMS ** (1 / 3))
    out = np.empty((n_walkers, n_atoms, 3))
    for w in range(n_walkers):
        rng = np.random.default_rng([2028, first + w])
        out[w] = sites * a + rng.normal(0.0, 0.03, size=(n_atoms, 3))
    return out, np.diag([a * m] * 3)


def accuracy_against(ref, got, pairs_ref=None, pairs_got=None):
    """Errors of one walker's GPU result against the FP64 oracle's: |dCV|/CV, the norm-wise
    max_i |dF_i| / max_i |F_i| of the derivatives, max |dvirial| / max |virial|, and whether the
    neighbour-list pair sets are identical."""
    s0, d0, v0 = ref
    s1, d1, v1 = got
    fn = np.sqrt((d0 ** 2).sum(axis=1)).max()
    out = {"cv_rel": abs(s1 - s0) / abs(s0),
           "force_rel_normwise": float(np.sqrt(((d1 - d0) ** 2).sum(axis=1)).max() / fn),
           "virial_rel": float(np.abs(np.asarray(v1).reshape(9) - np.asarray(v0).reshape(9)).max() /
                               np.abs(np.asarray(v0)).max())}
    if pairs_ref is not None and pairs_got is not None:
        out["nl_bit_exact"] = bool(np.array_equal(pairs_ref, pairs_got))
    return out


def cpu_baseline(frames, box, budget_s=10.0, gpu_check=None):
    """The reference algorithm on this host's cores: classic neighbour list once
    (amortised over NL_STRIDE=10 steps) + the CoordinationBase pair loop.  The
    oracle also checks the GPU's results, untimed (gpu_check: walker -> {"mixed":
    (s, deriv, virial, sorted pairs), "fp64": (s, deriv, virial), "build_pos": the
    rebuild frame (frames[w]), "pos": the checked step's positions})."""
    import oracle
    oracle.build()
    orc = oracle.Oracle()
    pos = frames[0]
    n = len(pos)
    t0 = time.perf_counter()
    pairs = orc.nl_classic_cells(0, n, 0, pos, box, True, 0.8)
    t_build = time.perf_counter() - t0
    kind = "port"
    nthreads = orc.max_threads()
    reps, t_loop = 0, 0.0
    while t_loop < budget_s or reps == 0:
        t0 = time.perf_counter()
        orc.coordination(SPEC, pos, box, pairs, nthreads=nthreads)
        t_loop += time.perf_counter() - t0
        reps += 1
    per_step = t_loop / reps + t_build / 10.0
    out = {"value": len(pairs) / per_step, "unit": "pair-evals/s", "cores": nthreads, "kind": kind,
           "sample": "1 walker of %d atoms: classic NL build once (%.2f s, serial, amortised /10) + %d pair "
                     "loops over %d NL pairs (OpenMP, %d threads)" % (n, t_build, reps, len(pairs), nthreads),
           "ms_per_step": per_step * 1e3}
    # one thread, one pair loop (the reference's serial CoordinationBase loop)
    t0 = time.perf_counter()
    orc.coordination(SPEC, pos, box, pairs, nthreads=1)
    t1 = time.perf_counter() - t0
    out["one_thread"] = {"value": len(pairs) / (t1 + t_build / 10.0), "unit": "pair-evals/s",
                         "pair_loop_ms": t1 * 1e3, "build_ms_amortised": t_build / 10.0 * 1e3}
    if gpu_check:
        acc = {}
        for w, got in sorted(gpu_check.items()):
            # the list of the rebuild frame, evaluated at the checked step's positions
            pw = pairs if w == 0 else orc.nl_classic_cells(0, n, 0, got["build_pos"], box, True, 0.8)
            ref = orc.coordination(SPEC, got["pos"], box, pw, nthreads=nthreads)
            e = {"mixed": accuracy_against(ref, got["mixed"][:3], pw, got["mixed"][3])}
            if "fp64" in got:
                e["fp64"] = accuracy_against(ref, got["fp64"])
            acc["walker_%d" % w] = e
        out["accuracy"] = acc
    return out


def _time_calls(torch, fn, calls):
    """Device time per call of fn(k) for k in calls (CUDA events on the default stream, which the library's
    NULL-stream calls are ordered with)."""
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    for k in calls:
        fn(k)
    ev1.record()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) * 1e-3 / max(len(calls), 1)


def run_c0(dev, frames=10, cpu=True):
    """The reference's CPU-runnable case: 1,000 atoms (10^3 lattice at 0.30 nm, sigma 0.03, a 3.0 nm box),
    GROUPA=1-1000, SWITCH={RATIONAL R_0=0.30 D_0=0.0 NN=6 MM=12 D_MAX=1.0}, no list (499,500 pairs), ten
    frames each re-jittered.  One CV+force call per frame, as a driver makes it, for the FP64 drop-in and
    the mixed path."""
    import torch
    from plumed2_gb300 import _lib
    from plumed2_gb300 import frames as FR
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.30 D_0=0.0 NN=6 MM=12 D_MAX=1.0"
    xs = np.stack([FR.workload_c0(frame=f)[0] for f in range(frames)])
    box = FR.workload_c0()[1]
    tx = torch.tensor(xs, dtype=torch.float64, device=dev)
    s = torch.zeros(1, dtype=torch.float64, device=dev)
    der = torch.zeros(1000, 3, dtype=torch.float64, device=dev)
    vir = torch.zeros(9, dtype=torch.float64, device=dev)
    out = {"workload": "1,000 atoms, 10^3 jittered sc lattice at 0.30 nm in a 3.0 nm box, GROUPA=1-1000, %s, "
                       "no neighbour list, %d frames, one CV+force call per frame" % (spec, frames),
           "pairs_per_frame": 499500, "unit": "pair-evals/s"}
    for prec in ("fp64", "mixed"):
        c = Coordination("GROUPA=1-1000 SWITCH={%s}" % spec, precision=prec, device=dev.index or 0)
        call = lambda k: c.forward_device(tx[k % frames].data_ptr(), box[None], 1, s.data_ptr(), der.data_ptr(),
                                          vir.data_ptr(), step=k)
        for k in range(3):
            call(k)
        t = _time_calls(torch, call, list(range(3, 3 + 3 * frames)))
        out[prec] = {"us_per_frame": t * 1e6, "value": 499500 / t}
        c.close()
    if cpu:
        import oracle
        oracle.build()
        orc = oracle.Oracle()
        pairs = orc.all_pairs(0, 1000)
        ref = []
        t0 = time.perf_counter()
        for f in range(frames):
            ref.append(orc.coordination(spec, xs[f], box, pairs, nthreads=1))
        t1 = (time.perf_counter() - t0) / frames
        out["cpu_baseline"] = {"value": 499500 / t1, "unit": "pair-evals/s", "cores": 1, "kind": "port",
                               "sample": "the %d frames, serial pair loop" % frames, "us_per_frame": t1 * 1e6}
    return out


def run_c1(dev, steps=100, cpu=True):
    """The mixed-precision single-CV case: 32,768 atoms (32^3 lattice at 0.31 nm, sigma 0.03, a 9.92 nm box),
    GROUPA = the z < L/2 slab, GROUPB = the other, RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=1.2, NLIST
    NL_CUTOFF=1.4 NL_STRIDE=20, frames that move by Gaussian steps of 0.002 nm.  One CV+force call per
    frame on the device, mixed and FP64."""
    import torch
    from plumed2_gb300 import frames as FR
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=1.2"
    line = "GROUPA=1-16384 GROUPB=16385-32768 SWITCH={%s} NLIST NL_CUTOFF=1.4 NL_STRIDE=20" % spec
    xs, box = FR.workload_c1(n_frames=steps + 20)
    tx = torch.tensor(xs, dtype=torch.float64, device=dev)
    s = torch.zeros(1, dtype=torch.float64, device=dev)
    der = torch.zeros(32768, 3, dtype=torch.float64, device=dev)
    vir = torch.zeros(9, dtype=torch.float64, device=dev)
    out = {"workload": "32,768 atoms, 32^3 jittered sc lattice at 0.31 nm in a 9.92 nm box, two z slabs as "
                       "GROUPA/GROUPB, %s, NLIST NL_CUTOFF=1.4 NL_STRIDE=20, frames moving by 0.002 nm Gaussian "
                       "steps; one CV+force call per frame, steps 20..%d timed" % (spec, 19 + steps),
           "unit": "pair-evals/s"}
    for prec in ("mixed", "fp64"):
        c = Coordination(line, precision=prec, device=dev.index or 0)
        call = lambda k: c.forward_device(tx[k].data_ptr(), box[None], 1, s.data_ptr(), der.data_ptr(),
                                          vir.data_ptr(), step=k)
        for k in range(20):
            call(k)
        t = _time_calls(torch, call, list(range(20, 20 + steps)))
        # the list sizes of the timed steps (untimed replay: one size per rebuild interval)
        pairs = 0
        for k in range(20, 20 + steps):
            if k % 20 == 0 or k == 20:
                call(k)
                size = c.nl_size()
            pairs += size
        out[prec] = {"us_per_step": t * 1e6, "value": pairs / steps / t, "pairs_per_step": pairs / steps}
        c.close()
    if cpu:
        import oracle
        oracle.build()
        orc = oracle.Oracle()
        nth = orc.max_threads()
        t0 = time.perf_counter()
        nl = orc.nl_classic_cells(1, 16384, 16384, xs[20], box, True, 1.4)
        tb = time.perf_counter() - t0
        t0 = time.perf_counter()
        for k in range(20, 25):
            orc.coordination(spec, xs[k], box, nl, nthreads=nth)
        tl = (time.perf_counter() - t0) / 5
        out["cpu_baseline"] = {"value": len(nl) / (tl + tb / 20), "unit": "pair-evals/s", "cores": nth,
                               "kind": "port", "sample": "five steps' pair loops (OpenMP) + 1/20 of the list build"}
    return out


def run_c3(dev, steps=60, cpu=True):
    """The differentiation case: the C1 system (32,768 atoms in two slabs, NLIST NL_CUTOFF=1.4 NL_STRIDE=20,
    frames moving by 0.002 nm Gaussian steps) under a 500-hill METAD bias (heights 1.2, sigma 0.05 s0,
    centres uniform in [0.8 s0, 1.2 s0]): each step the CV with kept derivatives, the bias energy and dV/ds
    on the device (k_bias_hills), then the backward (forces and box gradient).  Mixed and FP64.  The
    forces are checked against central finite differences of the biased energy (h = 1e-6 nm) in
    tests/test_gpu_backward.py."""
    import torch
    from plumed2_gb300 import _lib
    from plumed2_gb300 import frames as FR
    from plumed2_gb300.action import Coordination
    spec = "RATIONAL R_0=0.35 NN=6 MM=12 D_MAX=1.2"
    line = "GROUPA=1-16384 GROUPB=16385-32768 SWITCH={%s} NLIST NL_CUTOFF=1.4 NL_STRIDE=20" % spec
    xs, box = FR.workload_c1(n_frames=steps + 20)
    tx = torch.tensor(xs, dtype=torch.float64, device=dev)
    s = torch.zeros(1, dtype=torch.float64, device=dev)
    vir = torch.zeros(9, dtype=torch.float64, device=dev)
    g = torch.zeros(1, dtype=torch.float64, device=dev)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    gpos = torch.zeros(32768, 3, dtype=torch.float64, device=dev)
    gbox = torch.zeros(9, dtype=torch.float64, device=dev)
    gpar = torch.zeros(2, dtype=torch.float64, device=dev)
    dpar = torch.zeros(2, dtype=torch.float64, device=dev)
    out = {"workload": "C1's 32,768-atom two-slab system over frames moving by 0.002 nm Gaussian steps, %s, NLIST "
                       "NL_CUTOFF=1.4 NL_STRIDE=20, a 500-hill METAD bias on the CV; per step the CV with kept "
                       "derivatives, the bias and dV/ds on the device, the backward (forces, box gradient, dV/dR_0 "
                       "and dV/dD_0); steps 20..%d timed" % (spec, 19 + steps), "unit": "steps/s"}
    for prec in ("mixed", "fp64"):
        c = Coordination(line, precision=prec, device=dev.index or 0)
        c.forward_device(tx[0].data_ptr(), box[None], 1, s.data_ptr(), 0, 0, step=0, flags=_lib.FLAG_NO_DERIV)
        torch.cuda.synchronize()
        s0 = s.item()
        gen = torch.Generator(device="cpu").manual_seed(3)
        centres = (s0 * (0.8 + 0.4 * torch.rand(1, 500, generator=gen, dtype=torch.float64))).to(dev)
        sigmas = torch.full((1, 500), 0.05 * s0, dtype=torch.float64, device=dev)
        heights = torch.full((1, 500), 1.2, dtype=torch.float64, device=dev)

        def step(k):
            c.forward_device(tx[k].data_ptr(), box[None], 1, s.data_ptr(), 0, vir.data_ptr(), step=k,
                             flags=_lib.FLAG_SAVE | _lib.FLAG_DR0, dparam_ptr=dpar.data_ptr())
            _lib.bias_hills(1, s.data_ptr(), 500, centres.data_ptr(), sigmas.data_ptr(), heights.data_ptr(),
                            energy.data_ptr(), g.data_ptr())
            c.backward_device(tx[k].data_ptr(), box[None], 1, g.data_ptr(), gpos.data_ptr(), gbox.data_ptr(),
                              gpar.data_ptr())

        for k in range(20):
            step(k)
        t = _time_calls(torch, step, list(range(20, 20 + steps)))
        out[prec] = {"us_per_step": t * 1e6, "value": 1.0 / t}
        c.close()
    if cpu:
        import oracle
        oracle.build()
        orc = oracle.Oracle()
        nth = orc.max_threads()
        t0 = time.perf_counter()
        nl = orc.nl_classic_cells(1, 16384, 16384, xs[20], box, True, 1.4)
        tb = time.perf_counter() - t0
        t0 = time.perf_counter()
        for k in range(20, 25):
            orc.coordination(spec, xs[k], box, nl, nthreads=nth)
        tl = (time.perf_counter() - t0) / 5
        out["cpu_baseline"] = {"value": 1.0 / (tl + tb / 20), "unit": "steps/s", "cores": nth, "kind": "port",
                               "sample": "five steps' CV and derivative loops (OpenMP) + 1/20 of the list build; "
                                         "the bias on one CV costs nothing beside them"}
    return out


def run_c2(dev, steps=3, warmup=2, frames_per_launch=64, cpu=True):
    """The batched uneven-actions workload: 256 single-list COORDINATION actions over one
    100,000-atom system (GROUPA sizes log-uniform in [16, 4096], R_0 ~ U(0.25, 0.45), NN=6 MM=12
    D_MAX=1.0, no list), mixed precision, 64 frames per launch through one coord_multi batch
    replayed as a captured CUDA graph.  Returns the measured figures (pair-evals/s over the
    timed replays, CUDA events on the batch's stream)."""
    import ctypes as C
    import torch
    from plumed2_gb300 import _lib
    from plumed2_gb300 import frames as FR
    from plumed2_gb300.action import Coordination
    L = _lib.load()
    pos, box = FR.workload_c2_system()
    sizes, starts, r0 = FR.workload_c2_actions(256)
    specs = ["RATIONAL R_0=%.6f NN=6 MM=12 D_MAX=1.0" % x for x in r0]
    acts = [Coordination("GROUPA=%d-%d SWITCH={%s}" % (st + 1, st + sz, sp), precision="mixed")
            for sz, st, sp in zip(sizes, starts, specs)]
    for a in acts:
        a._ensure_groups()
    arr = (C.c_void_p * len(acts))(*[a._ctx.value for a in acts])
    m = C.c_void_p()
    if L.coord_multi_create(arr, len(acts), len(pos), C.byref(m)) != 0:
        raise RuntimeError(L.coord_multi_last_error(m).decode())
    per = C.c_int64()
    o = C.c_int64()
    L.coord_multi_deriv_offset(m, 0, C.byref(o), C.byref(per))
    F = frames_per_launch
    # frame f: the system moved by f Gaussian steps of 0.002 nm
    rng = np.random.default_rng(77)
    fr = np.empty((F,) + pos.shape)
    fr[0] = pos
    for f in range(1, F):
        fr[f] = fr[f - 1] + rng.normal(0.0, 0.002, size=pos.shape)
    tpos = torch.tensor(fr, dtype=torch.float64, device=dev)
    s = torch.zeros(F, len(acts), dtype=torch.float64, device=dev)
    der = torch.zeros(F, per.value, dtype=torch.float64, device=dev)
    vir = torch.zeros(F, len(acts), 9, dtype=torch.float64, device=dev)
    boxes = np.ascontiguousarray(np.stack([box] * F).reshape(F, 9))
    stream = torch.cuda.Stream(device=dev)
    L.coord_multi_use_graph(m, 1)
    args = (m, F, C.c_void_p(tpos.data_ptr()), boxes.ctypes.data_as(C.POINTER(C.c_double)), 0,
            C.c_void_p(s.data_ptr()), C.c_void_p(der.data_ptr()), C.c_void_p(vir.data_ptr()),
            C.c_void_p(stream.cuda_stream))
    for _ in range(warmup):
        if L.coord_multi_forward_device(*args) != 0:
            raise RuntimeError(L.coord_multi_last_error(m).decode())
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = _lib.launch_count()
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(steps):
            L.coord_multi_forward_device(*args)
        ev1.record(stream)
    torch.cuda.synchronize()
    t = ev0.elapsed_time(ev1) * 1e-3 / steps
    pairs_frame = int(sum(int(n) * (int(n) - 1) // 2 for n in sizes))
    pairs = pairs_frame * F
    out = {"workload": "100,000-atom jittered sc lattice (14.5 nm box), 256 single-list actions, GROUPA sizes "
                       "log-uniform in [16, 4096], R_0 ~ U(0.25, 0.45), NN=6 MM=12 D_MAX=1.0, no list, mixed "
                       "precision, %d frames per launch, one captured CUDA graph per launch" % F,
           "value": pairs / t, "unit": "pair-evals/s", "ms_per_launch": t * 1e3, "pairs_per_launch": pairs,
           "us_per_frame": t / F * 1e6, "launches_per_replay": (_lib.launch_count() - l0) / steps,
           "fp32": {"achieved_tflops": pairs * ALG_FLOPS_PER_PAIR / t / 1e12}}
    if cpu:
        # the reference algorithm on the host cores: every action's pair loop on one frame
        import oracle
        oracle.build()
        orc = oracle.Oracle()
        nth = orc.max_threads()
        t0 = time.perf_counter()
        s_ref = []
        for sz, st, sp in zip(sizes, starts, specs):
            sz, st = int(sz), int(st)
            s_ref.append(orc.coordination(sp, pos[st:st + sz], box, orc.all_pairs(0, sz), nthreads=nth)[0])
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": pairs_frame / tc, "unit": "pair-evals/s", "cores": nth, "kind": "port",
                               "sample": "one frame of the 256 actions (%d pairs), OpenMP pair loops" % pairs_frame}
        s0 = s[0].cpu().numpy()
        out["accuracy"] = {"cv_rel_max_over_actions": float(np.max(np.abs(s0 - np.array(s_ref)) / np.abs(s_ref)))}
    L.coord_multi_destroy(m)
    for a in acts:
        a.close()
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build()
    orc = oracle.Oracle()
    kind = "port"
    n = args.atoms if not args.quick else 32768
    frames, box = make_walkers(1, n, 0)
    pos = frames[0]
    nthreads = orc.max_threads()
    # Each timed step is charged its pair loop plus a tenth of the latest list
    # build (NL_STRIDE=10), so the figure does not depend on how many rebuilds
    # fall inside the timed window.  The build is the port's classic list
    # (NLIST: every pair within NL_CUTOFF by the reference's exact test,
    # NeighborList.cpp:237-308) found through link cells on one thread
    # (orc_nl_classic_cells), which gives the same pair set as the reference's
    # loop over all N(N-1)/2 candidates in a small fraction of its time.  The
    # reference's own code (oracle/_ref) builds a list inside every call, so it
    # pins the port in the tests rather than being timed here.
    pairs = None
    t_build = 0.0
    total_pairs, total_t, step = 0, 0.0, 0
    for it in range(args.warmup + args.steps):
        if pairs is None or step % 10 == 0:
            t0 = time.perf_counter()
            pairs = orc.nl_classic_cells(0, n, 0, pos, box, True, 0.8)
            t_build = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.coordination(SPEC, pos, box, pairs, nthreads=nthreads)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            total_pairs += len(pairs)
            total_t += dt + t_build / 10.0
        step += 1
    v = total_pairs / total_t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "pair-evals/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "1 walker per step of %d atoms, single list, %s, NLIST NL_CUTOFF=0.8 "
                                   "NL_STRIDE=10 (rebuild every 10th step)" % (n, SPEC)},
            "cpu_baseline": {"value": v, "unit": "pair-evals/s", "cores": nthreads, "kind": kind,
                             "sample": "%d walker-steps of %d atoms, %d NL pairs each, each step charged its "
                                       "pair loop + 1/10 of the serial list build (%.2f s)"
                                       % (args.steps, n, len(pairs), t_build)},
            "e2e": {"value": v, "unit": "pair-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from plumed2_gb300 import _lib
    from plumed2_gb300.action import Coordination

    W = args.walkers
    n = args.atoms if not args.quick else 32768
    frames, box = make_walkers(W, n, rank_walkers(rank, W)[0])
    boxes = np.stack([box] * W)
    line = LINE % (n, SPEC)
    c = Coordination(line, precision="mixed", device=local)
    # a trajectory per walker: the lattice frame, then Gaussian steps of MOTION_SIGMA per coordinate; step k
    # uses frame k % 10, so every rebuild (NL_STRIDE = 10) starts from the lattice frame and the nine steps
    # after it move away from it as an MD run does
    T = 10
    traj = torch.empty((T, W, n, 3), dtype=torch.float64, device=dev)
    traj[0] = torch.from_numpy(frames).to(dev)
    gen_t = torch.Generator(device=dev).manual_seed(11)
    for k in range(1, T):
        traj[k] = traj[k - 1] + MOTION_SIGMA * torch.randn((W, n, 3), generator=gen_t, dtype=torch.float64,
                                                            device=dev)

    def pos_ptr(st):
        return traj[st % T].data_ptr()

    s = torch.zeros(W, dtype=torch.float64, device=dev)
    der = torch.zeros(W, n, 3, dtype=torch.float64, device=dev)
    vir = torch.zeros(W, 9, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    step = 0
    # a metadynamics bias per walker: 500 METAD hills (truncated, stretched Gaussians, coord_bias_hills),
    # h = 1.2, sigma = 0.05 s0, centres uniform in [0.8 s0, 1.2 s0], s0 = the walker's first CV
    c.forward_device(pos_ptr(0), boxes, W, s.data_ptr(), 0, 0, step=0, flags=_lib.FLAG_NO_DERIV)
    torch.cuda.synchronize()
    s0 = s.clone()
    gen = torch.Generator(device="cpu").manual_seed(7)
    centres = (s0.cpu()[:, None] * (0.8 + 0.4 * torch.rand(W, 500, generator=gen, dtype=torch.float64))).to(dev)
    sigmas = (0.05 * s0[:, None]).expand(W, 500).contiguous()
    heights = torch.full((W, 500), 1.2, dtype=torch.float64, device=dev)
    g = torch.zeros(W, dtype=torch.float64, device=dev)
    gpos = torch.zeros(W, n, 3, dtype=torch.float64, device=dev)
    gbox = torch.zeros(W, 9, dtype=torch.float64, device=dev)
    energy = torch.zeros(W, dtype=torch.float64, device=dev)

    def one_step(ctx):
        """CV (derivatives and virial kept for backward) -> METAD hills bias energy and dV/ds on the device ->
        backward kernel: forces and the box gradient (what a metadynamics step needs)."""
        nonlocal step
        ctx.forward_device(pos_ptr(step), boxes, W, s.data_ptr(), 0, vir.data_ptr(), step=step,
                           flags=_lib.FLAG_SAVE)
        _lib.bias_hills(W, s.data_ptr(), 500, centres.data_ptr(), sigmas.data_ptr(), heights.data_ptr(),
                        energy.data_ptr(), g.data_ptr())
        ctx.backward_device(pos_ptr(step), boxes, W, g.data_ptr(), gpos.data_ptr(), gbox.data_ptr(), 0)
        step += 1

    for _ in range(args.warmup):
        one_step(c)
    torch.cuda.synchronize()
    pairs_per_step = sum(c.nl_size(w) for w in range(W))

    # timed region (events on the library's stream through a default-stream sync)
    clocks = Clocks(local)
    c.set_timing(True)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    clocks.start()
    # device time: CUDA events on the default stream, which the library's calls
    # with a NULL stream are fenced against on both sides
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        one_step(c)
    ev1.record()
    torch.cuda.synchronize()
    t = ev0.elapsed_time(ev1) * 1e-3
    clk = clocks.stop()
    launches = _lib.launch_count() - l0
    ktimes = c.kernel_times()
    kern_ms, kern_n = c.kernel_ms()
    c.set_timing(False)
    # the lists' near parts after the timed steps (what a step reads while the walkers stay within half
    # the skin of the rebuild), against their full size
    near = [c.nl_near_size(w) for w in range(W)]
    near_info = {"near_entries": sum(x[0] for x in near), "list_entries": sum(c.nl_size(w) for w in range(W)),
                 "skin_nm": near[0][1]}
    t = reduce_over_ranks(t, "max", dev)
    pairs_job = reduce_over_ranks(pairs_per_step, "sum", dev)
    ms_step = t / args.steps * 1e3
    value = pairs_job * args.steps / t

    # cost of one neighbour-list rebuild (at the next multiple of NL_STRIDE, the lattice frame) against a
    # plain CV+force pass, and the CV+force pass alone (s, ds/dx, virial: CoordinationBase::calculate) over
    # the five steps after it
    torch.cuda.synchronize()
    R = (step // T + 1) * T
    ev0.record()
    c.forward_device(pos_ptr(R), boxes, W, s.data_ptr(), der.data_ptr(), vir.data_ptr(), step=R,
                     flags=_lib.FLAG_REBUILD)
    ev1.record()
    torch.cuda.synchronize()
    t_rebuild_step = ev0.elapsed_time(ev1) * 1e-3
    ev0.record()
    for k in range(1, 6):
        c.forward_device(pos_ptr(R + k), boxes, W, s.data_ptr(), der.data_ptr(), vir.data_ptr(), step=R + k)
    ev1.record()
    torch.cuda.synchronize()
    t_plain_step = ev0.elapsed_time(ev1) * 1e-3 / 5
    # the mixed results of the last of those steps (R + 5: the list of the lattice frame, the walkers five
    # steps away from it) for two walkers, checked against the FP64 oracle in the CPU-baseline leg; and the
    # run-to-run spread of the derivative reduction: the same step again (its vector atomics add in
    # whatever order the hardware takes)
    check_w = sorted({0, W - 1})
    gpu_check = {}
    for w in check_w:
        p_ = np.asarray(c.pairs(w)).reshape(-1, 2)
        gpu_check[w] = {"mixed": (s[w].item(), der[w].cpu().numpy(), vir[w].cpu().numpy(),
                                  p_[np.lexsort((p_[:, 1], p_[:, 0]))]),
                        "build_pos": traj[0, w].cpu().numpy(), "pos": traj[5, w].cpu().numpy()}
    der_a = der.clone()
    s_a = s.clone()
    c.forward_device(pos_ptr(R + 5), boxes, W, s.data_ptr(), der.data_ptr(), vir.data_ptr(), step=R + 5)
    torch.cuda.synchronize()
    spread = {"deriv_max_abs_diff_rel": float((der - der_a).abs().max().item() / der_a.abs().max().item()),
              "cv_max_abs_diff_rel": float(((s - s_a).abs() / s_a.abs()).max().item()),
              "what": "the same mixed CV+force pass run twice on the same inputs, all walkers"}

    # the plain FP64 GPU path on the same workload (the drop-in, for the 5x target)
    c64 = Coordination(line, precision="fp64", device=local)
    c64.forward_device(pos_ptr(R), boxes, W, s.data_ptr(), der.data_ptr(), vir.data_ptr(), step=R)
    torch.cuda.synchronize()
    ev0.record()
    for k in range(1, 1 + args.fp64_steps):
        c64.forward_device(pos_ptr(R + k), boxes, W, s.data_ptr(), der.data_ptr(), vir.data_ptr(), step=R + k)
    ev1.record()
    torch.cuda.synchronize()
    t64 = ev0.elapsed_time(ev1) * 1e-3 / max(args.fp64_steps, 1)
    if args.fp64_steps != 5:  # the checked step, R + 5
        c64.forward_device(pos_ptr(R + 5), boxes, W, s.data_ptr(), der.data_ptr(), vir.data_ptr(), step=R + 5)
        torch.cuda.synchronize()
    for w in check_w:
        gpu_check[w]["fp64"] = (s[w].item(), der[w].cpu().numpy(), vir[w].cpu().numpy())
    c64.close()

    line_out = None
    if rank == 0:
        peaks = _lib.measure_peaks(local)
        mp = {}
        try:
            mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        hbm_peak = mp.get("hbm_gbs") or peaks["hbm_gbs"]
        # roofline of the pair kernel: algorithmic FLOPs and bytes per launch.  The launches read the rows' near
        # parts (the far entries are exactly zero while every atom is within half the skin of the rebuild):
        # per entry read one 4-byte list entry and one distance, per row a fixed-point position and an FP32
        # accumulator (read and written)
        pairs_launch = near_info["near_entries"] or pairs_per_step
        flops = pairs_launch * ALG_FLOPS_PER_PAIR
        bytes_alg = 4 * pairs_launch + 16 * W * n + 16 * W * n  # ELL entry + fixed-point positions + FP32 deriv accum
        achieved_tf = flops / (kern_ms * 1e-3) / 1e12 if kern_ms > 0 else None
        achieved_gbs = bytes_alg / (kern_ms * 1e-3) / 1e9 if kern_ms > 0 else None
        frac_fp32 = achieved_tf / peaks["fp32_tflops"] if achieved_tf else None
        frac_hbm = achieved_gbs / hbm_peak if achieved_gbs else None
        # the stored-list pair pass has no tensor-core work: its roof is HBM (the
        # list stream); the FP32 pipe's fraction is reported beside it
        # the pair-list layout's own count above; the count for a list of two
        # 4-byte indices per pair with FP32 derivatives (16 N + 8 P + 12 N)
        # beside it, for comparison
        bytes_2idx = 8 * pairs_per_step + 16 * W * n + 12 * W * n  # every list pair, as the reference's loop
        gbs_2idx = bytes_2idx / (kern_ms * 1e-3) / 1e9 if kern_ms > 0 else None
        roof = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": frac_hbm,
                "traffic": None,
                "alg_bytes_basis": "4 B per list entry read (one half-list entry: partner rank + orientation bit; "
                                   "the launches read the %d entries of the rows' near parts) + 16 B fixed-point "
                                   "position + 16 B FP32 accumulator per atom" % pairs_launch,
                "two_index_list": {"bytes_per_launch": bytes_2idx, "achieved": gbs_2idx,
                                   "frac": gbs_2idx / hbm_peak if gbs_2idx else None,
                                   "basis": "16 B/atom positions + 8 B/pair (two 4-byte indices) "
                                            "+ 12 B/atom FP32 derivatives, over every list pair (%d; the "
                                            "far ones are known to be zero without being read)"
                                            % pairs_per_step},
                "peak_source": ("MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)" if mp.get("hbm_gbs")
                                else "coord_measure_peaks copy microbenchmark (measured live)")}
        roof["traffic"] = eval_traffic(bytes_alg)
        roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at 16 x 110,592 "
                                  "atoms (profiles/k_eval_nl32_110592atoms_16walkers.md), scaled by the ratio of "
                                  "algorithmic bytes")
        kt = sorted(ktimes) or [0.0]
        roof.update({"kernel": "k_eval_nl32 (mixed NL pair kernel)", "kernel_ms": kern_ms, "launches": kern_n,
                     "kernel_ms_min_median_max": [kt[0], kt[len(kt) // 2], kt[-1]],
                     "fp64_peak_tflops": peaks["fp64_tflops"], "hbm_microbench_gbs": peaks["hbm_gbs"],
                     "alg_flops_per_launch": flops, "alg_bytes_per_launch": bytes_alg,
                     "fp32": {"achieved_tflops": achieved_tf, "peak_tflops": peaks["fp32_tflops"], "frac": frac_fp32,
                              "peak_source": "coord_measure_peaks FP32 FMA microbenchmark (measured live)"}})

        # e2e through the plugin-facing host call, one context per walker
        e2e_v, h2d, d2h = None, 0, 0
        pageable, tables = _lib.host_memory_access(local)
        host_path = ("direct: kernels read the positions from and write s, virial and forces into the caller's "
                     "host arrays through the host page tables" if pageable and tables and
                     os.environ.get("COORD_HOST_STAGED") != "1" else "staged through pinned host buffers")
        e2e_walker = None
        if args.e2e_steps > 0:
            from plumed2_gb300._lib import addr
            pin = lambda *shape: torch.empty(*shape, dtype=torch.float64, pin_memory=True).numpy()
            # the trajectory's frames in page-locked host memory, one per step of the stride
            hp, hs, hd, hv = pin(T, W, n, 3), pin(W), pin(W, n, 3), pin(W, 9)
            hp[:] = traj.cpu().numpy()
            e2e_v, e2e_windows, batch_paths, e2e_walker, walker_windows, walker_paths = measure_e2e(
                lambda: Coordination(line, precision="mixed", device=local), hp, hs, hd, hv, box, W, n,
                args.e2e_steps, addr)
            h2d = W * n * 3 * 8
            d2h = W * (n * 3 * 8 + 10 * 8)
        cpu = None
        if not args.no_cpu_baseline:
            cpu = cpu_baseline(frames, box, budget_s=8.0, gpu_check=gpu_check)
        c2 = c0 = c1 = c3 = None
        if args.c2_steps > 0:
            c2 = run_c2(dev, steps=args.c2_steps, cpu=not args.no_cpu_baseline)
            c0 = run_c0(dev, cpu=not args.no_cpu_baseline)
            c1 = run_c1(dev, cpu=not args.no_cpu_baseline)
            c3 = run_c3(dev, cpu=not args.no_cpu_baseline)
        line_out = {
            "metric": METRIC, "value": value, "unit": "pair-evals/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "262144-atom jittered sc lattice, 19.87 nm periodic box, single list, %s, NLIST "
                                   "NL_CUTOFF=0.8 NL_STRIDE=10, %d walkers per GPU batched per launch, mixed "
                                   "precision (FP32 pairs, FP64 compensated sums)" % (SPEC, W),
                       "atoms": n, "walkers_per_gpu": W, "pairs_per_step_per_gpu": pairs_per_step,
                       "us_per_step": ms_step * 1e3, "us_per_walker_step": ms_step * 1e3 / W,
                       "fp64_gpu_ms_per_step": t64 * 1e3,
                       "rebuild_step_ms": t_rebuild_step * 1e3,
                       "mixed_over_fp64_speedup_cv_force": t64 / t_plain_step,
                       "step": "CV with saved derivatives and virial + 500-hill METAD bias (device kernel) + "
                               "backward kernel (forces and box gradient) for all walkers; NL rebuilt every 10th step",
                       "cv_force_pass_ms": t_plain_step * 1e3, "autotune": c.autotune(),
                       "backward": True, "l2": "working set (0.8 GB) larger than the 129 MB L2",
                       "motion": "each walker moves by Gaussian steps of %g nm per coordinate per step; step k "
                                 "uses frame k %% 10, so every rebuild starts from the lattice frame" % MOTION_SIGMA,
                       "near_parts": dict(near_info, what="entries within D_MAX + skin at the last rebuild: a step "
                                                          "reads only these while every atom has moved less than "
                                                          "half the skin since it (far entries are then exactly "
                                                          "zero); value counts every list entry, as the "
                                                          "reference's loop does"),
                       "parallelism": "walkers sharded across GPUs, no collective"},
            "roofline": roof, "cpu_baseline": cpu,
            "accuracy": dict((cpu or {}).get("accuracy", {}), run_to_run=spread,
                             basis="the CV+force pass of a non-rebuild step against the FP64 oracle "
                                   "(oracle/, the C restatement pinned to the reference) on the same positions "
                                   "and the same neighbour list; targets |dCV|/CV <= 1e-6, force <= 1e-5 "
                                   "(norm-wise), bit-exact list"),
            "e2e": {"value": e2e_v, "unit": "pair-evals/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "call": "coord_forward_batch (C ABI, pinned host arrays of all %d walkers by address): the "
                            "median of %d windows of %d steps from step 11 on, each ending on a rebuild step (lists "
                            "rebuilt on multiples of 10), after eleven untimed steps"
                            % (W, E2E_WINDOWS, args.e2e_steps),
                    "windows": e2e_windows if args.e2e_steps > 0 else None,
                    "host_path": host_path_note(batch_paths) if args.e2e_steps > 0 else None,
                    "per_walker_call": {"value": e2e_walker, "unit": "pair-evals/s",
                                        "call": "coord_forward per walker and step (the plugin's call), one context "
                                                "per walker, pageable host arrays: one position array per walker "
                                                "rewritten in place between steps (untimed), as an MD engine does; "
                                                "the median of %d windows of %d steps from step 11 on, after ten "
                                                "untimed steps" % (E2E_WINDOWS, args.e2e_steps),
                                        "windows": walker_windows if args.e2e_steps > 0 else None,
                                        "host_path": host_path_note(walker_paths) if args.e2e_steps > 0
                                        else host_path}},
            "gpu_launches": launches, "clocks": clk,
            "other_configs": {"c2_batched_uneven_actions": c2, "c0_cpu_case": c0, "c1_mixed_single_cv": c1,
                              "c3_metad_backward": c3},
        }
        print(json.dumps(line_out), flush=True)
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in ("c3", "c2", "c1", "c0"):
        import torch
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        if args.workload == "c2":
            out = run_c2(dev, steps=args.steps, warmup=args.warmup, cpu=not args.no_cpu_baseline)
        elif args.workload == "c1":
            out = run_c1(dev, steps=args.steps, cpu=not args.no_cpu_baseline)
        elif args.workload == "c3":
            out = run_c3(dev, steps=args.steps, cpu=not args.no_cpu_baseline)
        else:
            out = run_c0(dev, cpu=not args.no_cpu_baseline)
        print(json.dumps(dict(out, metric=METRIC, n_gpus=1, steps=args.steps, warmup=args.warmup,
                              higher_is_better=True, dtype="f32", data="synthetic")), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

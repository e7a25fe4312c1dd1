"""Benchmark of the batched alignment solve on GB300 (one JSON line on stdout).

Workload (the batched form of pyalign's ProblemBatch solve): local alignment
(Smith-Waterman) with affine gaps (Gotoh, open 5, extend 2), DNA alphabet {A,C,G,T}
i.i.d. uniform, match +2 / mismatch -3 (int32 scores), 65,536 pairs whose lengths are drawn
independently uniform in [100, 1000]; half of the pairs are a seeded query and a copy of it
with 10% random substitutions/insertions/deletions.  Codomain: score plus one optimal
traceback per pair (pyalign.solve.LocalSolver(AffineGapCost(5, 2), codomain=Alignment)).
Data is synthetic and seeded (no dataset involved).

A "step" is one pass of the solve over the whole batch.  `value` is GCUPS (cells = sum of
|s|*|t|) with the codes already resident in HBM; `e2e` is the same metric through the C ABI
with pinned host buffers, host<->device copies inside the timed region.  The reference arm
(--impl reference) times the CPU restatement of the reference's solver (the reference's
xtensor core cannot be built here) on the host cores.
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

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

METRIC = "GCUPS: batched Gotoh score+traceback, and fwd+bwd, vs plain GPU path, 1 GB300"
WORKLOAD = "local affine (Gotoh 5/2) DNA +2/-3, 65536 pairs, |s|,|t| ~ U[100,1000], score + one traceback"
# algorithmic ALU ops per cell: Gotoh 9 + local zero 1 + one-optimal traceback mask 4
OPS_PER_CELL = 14
# algorithmic HBM bytes per cell: the 4-bit traceback nibble
BYTES_PER_CELL = 0.5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs", type=int, default=65536)
    ap.add_argument("--seed", type=int, default=1002)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU work of the baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fwd-bwd-pairs", type=int, default=4096, help="pairs of the fwd+bwd measurement (0: skip)")
    ap.add_argument("--other-configs", type=int, default=1, help="also measure the other workloads (0: skip)")
    ap.add_argument("--precision-pairs", type=int, default=8192, help="pairs of the precision measurement (0: skip)")
    ap.add_argument("--prepare", type=int, default=1, help="also time problem preparation from strings (0: skip)")
    ap.add_argument("--allopt-pairs", type=int, default=256,
                    help="pairs of 5000 x 10000 in the all-optimal measurement of the long-pair workload")
    ap.add_argument("--plain", type=int, default=1,
                    help="also time the plain GPU path: one launch per 100-wide length bucket (0: skip)")
    ap.add_argument("--plain-pairs", type=int, default=None,
                    help="earlier spelling of --plain (0 skips the plain path)")
    args = ap.parse_args()
    if args.plain_pairs is not None:
        args.plain = int(args.plain_pairs != 0)
    return args


# --------------------------------------------------------------------------- workload

def mutate(rng, s, rate=0.1, alphabet=4):
    """Copy of s with `rate` events per position: substitution / insertion / deletion."""
    n = len(s)
    ev = rng.random(n) < rate
    kind = rng.integers(0, 3, n)
    out = s.copy()
    sub = ev & (kind == 0)
    out[sub] = rng.integers(0, alphabet, int(sub.sum()))
    ins = ev & (kind == 1)
    keep = ~(ev & (kind == 2))
    counts = keep.astype(np.int64) + ins.astype(np.int64)
    idx = np.repeat(np.arange(n), counts)
    vals = out[idx]
    first = np.cumsum(counts) - counts
    vals[first[ins]] = rng.integers(0, alphabet, int(ins.sum()))
    return vals.astype(np.uint32)


def make_workload(pairs, seed, lo=100, hi=1000):
    rng = np.random.default_rng(seed)
    ls = rng.integers(lo, hi + 1, size=pairs).astype(np.int32)
    lt = rng.integers(lo, hi + 1, size=pairs).astype(np.int32)
    a = rng.integers(0, 4, size=(pairs, hi), dtype=np.uint32)
    b = rng.integers(0, 4, size=(pairs, hi), dtype=np.uint32)
    related = rng.random(pairs) < 0.5
    for k in np.nonzero(related)[0]:
        t = mutate(rng, a[k, :ls[k]])
        if len(t) > hi:
            t = t[:hi]
        if len(t) < lo:
            t = np.concatenate([t, rng.integers(0, 4, lo - len(t)).astype(np.uint32)])
        b[k, :len(t)] = t
        lt[k] = len(t)
    for k in range(pairs):  # padding as the reference's forms leave it: zeros
        a[k, ls[k]:] = 0
        b[k, lt[k]:] = 0
    table = np.full((4, 4), -3.0, dtype=np.float32)
    np.fill_diagonal(table, 2.0)
    return a, b, ls, lt, table


class AffineGap:
    """pyalign.gaps.AffineGapCost(open, extend) as seen by the native module (gaps.py:164-193)."""

    def __init__(self, open_, extend):
        self.u, self.v = open_ - extend, extend

    def to_special_case(self):
        return {"affine": (self.u, self.v)}


def options_dict(alg, batch_size):
    import types
    return {
        "solver": alg.Type.ALIGNMENT, "direction": alg.Direction.MAXIMIZE, "batch": True,
        "batch_size": batch_size, "return_dup": False, "locality": alg.Locality.LOCAL,
        "codomain": types.SimpleNamespace(detail=alg.Detail.ALIGNMENT, count=alg.Count.ONE),
        "gap_cost": AffineGap(5.0, 2.0),
    }


# --------------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clock/throttle sampling (read-only) every 20 ms, started before the
    warm-up; each sample carries the host time it arrived, and a summary keeps only the
    samples inside the marked timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 20

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.samples = []          # (host monotonic time, line)
        self.regions = {}
        self.first = threading.Event()

    def __enter__(self):
        return self.start()

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            self.first.wait(timeout=10.0)   # nvidia-smi's start-up must not eat the timed region
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.monotonic(), line.strip()))
            self.first.set()

    def begin(self, name):
        self.regions[name] = [time.monotonic(), None]

    def end(self, name):
        self.regions[name][1] = time.monotonic()

    def __exit__(self, *exc):
        self.stop()

    def stop(self):
        if self.proc:
            time.sleep(2.0 * self.PERIOD_MS / 1000.0)   # the sample after the last mark
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, name):
        t0, t1 = self.regions.get(name, (None, None))
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, line in self.samples:
            if t0 is None or t1 is None or not (t0 <= t <= t1):
                continue
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
                pw.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0,
               "period_ms": self.PERIOD_MS, "window_s": None if t1 is None else t1 - t0}
        if sm:
            out.update({"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm), "sm_max_mhz": max(mx),
                        "power_w_median": statistics.median(pw), "reasons": sorted(reasons),
                        "samples": len(sm)})
        return out


# --------------------------------------------------------------------------- CPU baseline

def oracle_solver(oalg, locality, detail, gap, cap_s, cap_t):
    """An oracle solver (CPU restatement of the reference's solver) with the options the
    native module would receive for this workload."""
    import types
    return oalg.m16.create_solver(cap_s, cap_t, oalg.m16.create_options({
        "solver": oalg.Type.ALIGNMENT, "direction": oalg.Direction.MAXIMIZE, "batch": True, "batch_size": 1,
        "return_dup": False, "locality": oalg.Locality.__members__[locality],
        "codomain": types.SimpleNamespace(detail=oalg.Detail.__members__[detail], count=oalg.Count.ONE),
        "gap_cost": gap}))


def cpu_baseline(a, b, ls, lt, table, seconds, threads=None):
    """The oracle (CPU restatement of the reference's solver) on a bounded prefix of the
    workload: score + one alignment per pair, `threads` host threads (default: all).
    Returns (GCUPS, threads, sample description, pairs, scores, maps) -- the scores and the
    concatenated alignment maps of those pairs are the parity check of the GPU arm."""
    import oracle.algorithm as oalg
    threads = threads or os.cpu_count() or 1
    solver = oracle_solver(oalg, "LOCAL", "ALIGNMENT", AffineGap(5.0, 2.0), a.shape[1], b.shape[1])

    def run(n):
        t0 = time.perf_counter()
        sc, mp, _, cells = oalg.batch_alignments(solver, a[:n], b[:n], table, ls[:n], lt[:n], threads)
        return cells, time.perf_counter() - t0, sc, mp

    cells, dt, _, _ = run(min(len(ls), threads * 2))
    target = cells / max(dt, 1e-6) * seconds
    cum = np.cumsum(ls.astype(np.int64) * lt.astype(np.int64))
    n = int(np.searchsorted(cum, target)) + 1
    n = max(threads, min(n, len(ls)))
    cells, dt, sc, mp = run(n)
    return (cells / dt / 1e9, threads, f"first {n} pairs of the workload ({cells:.3e} cells, {dt:.1f} s)",
            n, sc, mp)


def parity_of(n, sc_ref, mp_ref, sc, mp):
    """Bit-exact comparison of the first n pairs' scores and concatenated alignment maps."""
    bad = int(np.count_nonzero(np.asarray(sc[:n]) != sc_ref[:n]))
    maps_equal = mp_ref is None or np.array_equal(np.asarray(mp[:len(mp_ref)]), mp_ref)
    return {"pairs": int(n), "score_mismatches": bad, "maps_equal": bool(maps_equal),
            "mismatches": bad + (0 if maps_equal else 1)}


# --------------------------------------------------------------------------- other workloads

def _time_device(torch, fn, steps=5, warmup=3):
    """Mean device time of fn over `steps` calls after `warmup` untimed ones (the first call
    plans, the second captures the repeat's CUDA graph)."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1000.0 / steps


def make_global_linear_64(seed, pairs=4096):
    """4096 pairs of 64 x 64 letters i.i.d. uniform over 20: global alignment, linear gap 1,
    eq +1 / ne -1 (pyalign's binary form)."""
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 20, size=(pairs, 64)).astype(np.uint32)
    b = rng.integers(0, 20, size=(pairs, 64)).astype(np.uint32)
    ln = np.full(pairs, 64, np.int32)
    return a, b, ln, ln.copy()


def make_semiglobal_long(seed, pairs=256, ls=5000, lt=10000):
    """256 pairs of 5000 x 10000 residues of a 20-letter alphabet with per-batch letter
    frequencies ~ Dirichlet(1) and a seeded symmetric integer substitution matrix (diagonal
    U[4, 11], off-diagonal U[-4, 2]): semiglobal alignment, affine gap open 10 / extend 1."""
    rng = np.random.default_rng(seed)
    freq = rng.dirichlet(np.ones(20))
    a = rng.choice(20, size=(pairs, ls), p=freq).astype(np.uint32)
    b = rng.choice(20, size=(pairs, lt), p=freq).astype(np.uint32)
    m = rng.integers(-4, 3, size=(20, 20))
    m = np.triu(m, 1) + np.triu(m, 1).T
    np.fill_diagonal(m, rng.integers(4, 12, size=20))
    return a, b, np.full(pairs, ls, np.int32), np.full(pairs, lt, np.int32), m.astype(np.float32)


class LogGap:
    """pyalign.gaps.LogarithmicGapCost(u, v) (w(k) = u + v ln k, gaps.py:195-225) as seen by the
    native module: a general cost vector."""

    def __init__(self, u, v):
        self.u, self.v = u, v

    def to_special_case(self):
        return {}

    def costs(self, n):
        w = np.full((n,), self.u, dtype=np.float32)
        w[1:] += self.v * np.log(np.arange(1, n), dtype=np.float32)
        w[0] = 0
        return w


class LinearGap:
    """pyalign.gaps.LinearGapCost(g) as seen by the native module (gaps.py:120-160)."""

    def __init__(self, g):
        self.g = g

    def to_special_case(self):
        return {"linear": self.g}


def other_configs(torch, alg, L, seed, allopt_pairs=256):
    """The other synthetic workloads of the solve, through pa_solve_batch / the native
    module with device-resident codes: (1) global linear gap 1, eq +1 / ne -1, 4096 pairs
    of 64 letters over 20, score + one traceback; (3) semiglobal affine open 10 / extend 1
    on 256 pairs of 5000 x 10000 residues of a 20-letter alphabet (per-batch Dirichlet(1)
    frequencies, symmetric integer matrix: diagonal U[4, 11], off-diagonal U[-4, 2]),
    score only, and all-optimal: masks, path counts and the first 20 alignments of every
    pair on the device."""
    import types
    out = {}
    P = ctypes.POINTER

    def run_batch(opts, a, b, ls, lt, table=None, eq=None, ne=None, maps=True):
        B = a.shape[0]
        mod = alg.m16 if max(a.shape[1], b.shape[1]) < 16000 else alg.m32
        solver = mod.create_solver(a.shape[1], b.shape[1], mod.create_options(opts))
        alg.check(L.pa_solver_set_stream(solver.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        a_d = torch.from_numpy(a.view(np.int32)).cuda()
        b_d = torch.from_numpy(b.view(np.int32)).cuda()
        t_d = torch.from_numpy(table).cuda() if table is not None else None
        length = np.ascontiguousarray(np.stack([ls, lt]), dtype=np.int32)
        sizes = np.minimum(ls, lt).astype(np.int64)
        offs = np.zeros(B, np.int64)
        offs[1:] = np.cumsum(sizes)[:-1]
        sc = torch.empty(B, dtype=torch.float32, device="cuda")
        mp = torch.empty(max(1, int(sizes.sum())), dtype=torch.int32, device="cuda")
        bt = alg.Batch(form=1 if table is not None else 2, location=1, batch=B, n_s=a.shape[1], n_t=b.shape[1],
                       a=ctypes.cast(a_d.data_ptr(), P(ctypes.c_uint32)), b=ctypes.cast(b_d.data_ptr(), P(ctypes.c_uint32)),
                       table=ctypes.cast(t_d.data_ptr(), P(ctypes.c_float)) if t_d is not None else None,
                       table_rows=table.shape[0] if table is not None else 0,
                       table_cols=table.shape[1] if table is not None else 0,
                       eq=eq or 0.0, ne=ne or 0.0, length=length.ctypes.data_as(P(ctypes.c_int32)))

        def step():
            alg.check(L.pa_solve_batch(solver.handle, ctypes.byref(bt), ctypes.c_void_p(sc.data_ptr()),
                                       ctypes.c_void_p(mp.data_ptr()) if maps else None,
                                       offs.ctypes.data_as(P(ctypes.c_int64))))
        t = _time_device(torch, step)
        ms4 = (ctypes.c_float * 4)()
        nl = ctypes.c_int32(0)
        L.pa_solver_last_timings(solver.handle, ms4, ctypes.byref(nl))
        cells = float((ls.astype(np.int64) * lt).sum())
        return {"value": cells / t / 1e9, "unit": "GCUPS", "ms": t * 1000, "dp_ms": ms4[1], "traceback_ms": ms4[2],
                "plan": solver.last_plan()}, sc.cpu().numpy(), mp.cpu().numpy()

    def opts(alg_, locality, detail, gap, batch, count="ONE"):
        return {"solver": alg_.Type.ALIGNMENT, "direction": alg_.Direction.MAXIMIZE, "batch": True,
                "batch_size": batch, "return_dup": False, "locality": alg_.Locality.__members__[locality],
                "codomain": types.SimpleNamespace(detail=alg_.Detail.__members__[detail], count=alg_.Count.__members__[count]),
                "gap_cost": gap}

    import oracle.algorithm as oalg   # the oracle that checks the sampled pairs' results

    # config 1: every pair against the oracle (eq/ne as a 20 x 20 table of the indexed form)
    a1, b1, l1, _ = make_global_linear_64(seed)
    B1 = a1.shape[0]
    r1, sc1, mp1 = run_batch(opts(alg, "GLOBAL", "ALIGNMENT", LinearGap(1.0), B1), a1, b1, l1, l1, eq=1.0, ne=-1.0)
    eqne = np.where(np.eye(20, dtype=bool), 1.0, -1.0).astype(np.float32)
    osol = oracle_solver(oalg, "GLOBAL", "ALIGNMENT", LinearGap(1.0), 64, 64)
    osc, omp, _, _ = oalg.batch_alignments(osol, a1, b1, eqne, l1, l1)
    out["global_linear_64x64"] = dict(
        r1, parity=parity_of(B1, osc, omp, sc1, mp1),
        workload="4096 pairs of 64 x 64, 20 letters, global linear gap 1, eq +1 / ne -1, score + one traceback")
    # config 3: score only; the first pairs of the bag against the oracle's two-row score
    a3, b3, ls3, lt3, t3 = make_semiglobal_long(seed + 1)
    B3 = a3.shape[0]
    r3, sc3, _ = run_batch(opts(alg, "SEMIGLOBAL", "SCORE", AffineGap(10.0, 1.0), B3), a3, b3, ls3, lt3, table=t3,
                           maps=False)
    n3 = 4
    osol = oracle_solver(oalg, "SEMIGLOBAL", "SCORE", AffineGap(10.0, 1.0), 5000, 10000)
    osc3, _ = oalg.batch_scores_lean(osol, a3[:n3], b3[:n3], t3, ls3[:n3], lt3[:n3])
    out["semiglobal_affine_5000x10000_score"] = dict(
        r3, parity=parity_of(n3, osc3, None, sc3, None),
        workload="256 pairs of 5000 x 10000, 20 letters, semiglobal affine 10/1, score only")
    # length buckets: half the pairs short queries against long targets, half long pairs (local
    # Gotoh 5/2, DNA +2/-3); the tuner's plan (a group width per length bucket of |s| where
    # that times faster) against the one width it would use otherwise, same results required
    rs = np.random.default_rng(seed + 5)
    nbk, hbk = 32768, 16384
    ls_b = np.concatenate([rs.integers(16, 49, hbk), rs.integers(600, 1001, nbk - hbk)])
    lt_b = np.concatenate([rs.integers(800, 1001, hbk), rs.integers(600, 1001, nbk - hbk)])
    a_b = rs.integers(0, 4, (nbk, 1000)).astype(np.uint32)
    b_b = rs.integers(0, 4, (nbk, 1000)).astype(np.uint32)
    t_b = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(t_b, 2.0)
    o_b = opts(alg, "LOCAL", "ALIGNMENT", AffineGap(5.0, 2.0), nbk)
    rb, scb, mpb = run_batch(o_b, a_b, b_b, ls_b, lt_b, table=t_b)
    saved = os.environ.get("PA_GROUP_WIDTH")
    os.environ["PA_GROUP_WIDTH"] = str(rb["plan"]["G"])
    try:
        ru, scu, mpu = run_batch(o_b, a_b, b_b, ls_b, lt_b, table=t_b)
    finally:
        if saved is None:
            os.environ.pop("PA_GROUP_WIDTH", None)
        else:
            os.environ["PA_GROUP_WIDTH"] = saved
    out["length_buckets_skewed"] = {
        "tuned": rb, "one_width": ru, "tuned_over_one_width": ru["dp_ms"] / rb["dp_ms"],
        "same_results": bool(np.array_equal(scb, scu) and np.array_equal(mpb, mpu)),
        "workload": f"{nbk} pairs: half |s| ~ U[16, 48] x |t| ~ U[800, 1000], half |s|, |t| ~ U[600, 1000]; "
                    "local Gotoh 5/2, DNA +2/-3, score + one traceback, device-resident codes"}
    del a_b, b_b
    # general (logarithmic) gap costs, O(|s| |t| (|s| + |t|)): 64 pairs of 300 x 300 DNA, local,
    # score + one alignment through the native module; the first pairs against the oracle
    rw = np.random.default_rng(seed + 3)
    Bw, Lw = 64, 300
    aw = rw.integers(0, 4, size=(Bw, Lw)).astype(np.uint32)
    bw = aw.copy()
    mut = rw.random(size=(Bw, Lw)) < 0.15
    bw[mut] = rw.integers(0, 4, size=int(mut.sum()))
    tw = np.full((4, 4), -3.0, np.float32)
    np.fill_diagonal(tw, 2.0)
    lnw = np.full((2, Bw), Lw, np.uint16)
    ow = opts(alg, "LOCAL", "ALIGNMENT", LogGap(3.0, 1.0), Bw)
    sw = alg.m16.create_solver(Lw, Lw, alg.m16.create_options(ow))
    resw = sw.solve_indexed_for_alignment(aw, bw, tw, lnw)
    torch.cuda.synchronize()
    calls_w, dp_w = [], []
    for _ in range(5):
        t0 = time.perf_counter()
        resw = sw.solve_indexed_for_alignment(aw, bw, tw, lnw)
        calls_w.append(time.perf_counter() - t0)
        dp_w.append(sw.last_timings()[0][1])
    t_w = float(np.median(calls_w))
    kw = 4
    osw = oracle_solver(oalg, "LOCAL", "ALIGNMENT", LogGap(3.0, 1.0), Lw, Lw)
    osc_w, omp_w, offs_w, _ = oalg.batch_alignments(osw, aw[:kw], bw[:kw], tw, np.full(kw, Lw), np.full(kw, Lw))
    gsc_w = np.array([resw[k].score for k in range(kw)], np.float32)
    gmp_w = np.concatenate([np.asarray(resw[k].s_to_t, np.int32) for k in range(kw)])
    cells_w = float(Bw * Lw * Lw)
    out["local_log_gap_300x300"] = {
        "value": cells_w / t_w / 1e9, "unit": "GCUPS", "ms": t_w * 1000, "dp_ms": float(np.median(dp_w)),
        "candidates_per_s": cells_w * (2 * Lw) / t_w,
        "dp_candidates_per_s": cells_w * (2 * Lw) / (float(np.median(dp_w)) / 1000), "plan": sw.last_plan(),
        "parity": parity_of(kw, osc_w, omp_w, gsc_w, gmp_w),
        "workload": "64 pairs of 300 x 300 DNA (a query and a 15%-substituted copy), local, general gap "
                    "3 + ln k, score + one alignment, host arrays through the native module; median of 5 calls, "
                    "dp_ms the general-gap kernel's CUDA-event time (a 2-CTA cluster per pair)"}

    # all-optimal codomain on the whole bag through the native module's iterator form:
    # one solve writes the 16-bit all-optimal masks of all 256 pairs (25.6 GB, left on the
    # device), the co-optimal path counts of every pair are computed on the device, the
    # first 20 alignments of every pair are enumerated on the device in the reference's
    # order, and the host search (pa_iterator_next) enumerates the first 20 of two pairs --
    # the reference's way, one lane at a time -- which must equal the device's
    mod = alg.m16
    Ba = min(allopt_pairs, B3)
    o3 = opts(alg, "SEMIGLOBAL", "ALIGNMENT", AffineGap(10.0, 1.0), Ba, count="ALL")
    solver = mod.create_solver(5000, 10000, mod.create_options(o3))
    ln3 = np.stack([ls3[:Ba], lt3[:Ba]]).astype(np.uint16)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = solver.solve_indexed_for_alignment_iterator(a3[:Ba], b3[:Ba], t3, ln3)
    t_solve = time.perf_counter() - t0
    ms4 = (ctypes.c_float * 4)()
    nl = ctypes.c_int32(0)
    L.pa_solver_last_timings(solver.handle, ms4, ctypes.byref(nl))
    allopt_phases = {"upload": ms4[0], "dp": ms4[1], "traceback": ms4[2], "download": ms4[3]}
    t0 = time.perf_counter()
    counts = alg.path_counts(res[0]._res)
    t_count = time.perf_counter() - t0
    t0 = time.perf_counter()
    first = alg.FirstAlignments(res[0]._res, 20)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    host_maps = []
    for lane in range(min(2, Ba)):
        h = ctypes.c_void_p()
        alg.check(L.pa_result_iterator(res[0]._res.ptr, lane, ctypes.byref(h)))
        for _ in range(20):
            mp = np.zeros(min(int(ls3[lane]), int(lt3[lane])), np.int32)
            if not L.pa_iterator_next(h, None, mp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), None, None):
                break
            host_maps.append((lane, mp))
        L.pa_iterator_destroy(h)
    t_enum = time.perf_counter() - t0
    seen = {}
    enum_bad = 0
    for lane, mp in host_maps:
        j = seen.get(lane, 0)
        seen[lane] = j + 1
        enum_bad += int(j >= first.counts[lane] or not np.array_equal(first.alignment(lane, j)[0], mp))
    enum_bad += sum(int(first.counts[lane]) != seen.get(lane, 0) for lane in range(min(2, Ba)))
    n_items = len(host_maps)
    del res
    cells3 = float((ls3[:Ba].astype(np.int64) * lt3[:Ba]).sum())
    out["semiglobal_affine_5000x10000_all_optimal"] = {
        "value": cells3 / t_solve / 1e9, "unit": "GCUPS", "ms": t_solve * 1000, "pairs": Ba,
        "mask_bytes": int(2 * cells3), "plan": solver.last_plan(), "phases_ms": allopt_phases,
        "path_counts": {"ms": t_count * 1000, "gcups": cells3 / t_count / 1e9,
                        "min": int(counts.min()), "median": float(np.median(counts.astype(np.float64))),
                        "max": int(counts.max()), "saturated": int((counts == np.iinfo(np.uint64).max).sum())},
        "first_alignments": {"pairs": Ba, "alignments": int(first.counts.sum()), "ms": t_dev * 1000,
                             "alignments_per_s": float(first.counts.sum()) / t_dev,
                             "host_search": {"pairs": min(2, Ba), "alignments": n_items, "ms": t_enum * 1000,
                                             "alignments_per_s": n_items / t_enum if t_enum > 0 else None},
                             "parity": {"compared": n_items, "mismatches": enum_bad,
                                        "against": "the host search (pa_iterator_next) of the same lanes"}},
        "workload": f"{Ba} pairs of 5000 x 10000, all-optimal masks of every pair on the GPU (host-timed solve "
                    "call), co-optimal path counts on the GPU, first 20 alignments of every pair enumerated on "
                    "the GPU (host-timed call, maps on the host), and of 2 pairs by the host search"}
    return out


# --------------------------------------------------------------------------- prepare

def prepare_config(torch, a, b, ls, lt, sample=8192):
    """Problem preparation of the bench bag from strings (pyalign's indexed form,
    solve.py:382-396): the reference's way -- each string encoded on its own through the
    alphabet's 256-entry byte index (ByteAlphabetEncoder.encode, factory.py:114-127),
    restated, timed on a sample of pairs and reported per pair -- against one batch call of
    pa_encode_latin1 into host rows and into device rows (one upload of the raw bytes)."""
    from pyalign_gb300 import prepare as prep
    letters = np.array(list("ACGT"))
    B = a.shape[0]
    s_list = ["".join(letters[a[k, :ls[k]]]) for k in range(B)]
    t_list = ["".join(letters[b[k, :lt[k]]]) for k in range(B)]
    lut = prep.lut_of("ACGT")
    n = min(sample, B)
    rows = np.zeros((n, a.shape[1]), np.uint32)
    t0 = time.perf_counter()
    for k in range(n):  # the per-problem encoder's work, string by string
        r = lut[np.frombuffer(s_list[k].encode("latin1"), dtype=np.uint8)]
        if np.max(r) == 0xFF:
            raise ValueError("item not in alphabet")
        rows[k, :len(r)] = r
        r = lut[np.frombuffer(t_list[k].encode("latin1"), dtype=np.uint8)]
        if np.max(r) == 0xFF:
            raise ValueError("item not in alphabet")
        rows[k, :len(r)] = r
    per_problem = (time.perf_counter() - t0) / n
    host_a = np.zeros(a.shape, np.uint32)
    host_b = np.zeros(b.shape, np.uint32)
    t0 = time.perf_counter()
    prep.encode_latin1(s_list, lut, out=host_a, width=a.shape[1])
    prep.encode_latin1(t_list, lut, out=host_b, width=b.shape[1])
    host_s = time.perf_counter() - t0
    if not (np.array_equal(host_a, a) and np.array_equal(host_b, b)):
        raise SystemExit("batch encoding differs from the bench codes")
    dev_a = torch.empty(a.shape, dtype=torch.int32, device="cuda")
    dev_b = torch.empty(b.shape, dtype=torch.int32, device="cuda")
    prep.encode_latin1(s_list[:64], lut, out=dev_a, width=a.shape[1])  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prep.encode_latin1(s_list, lut, out=dev_a, width=a.shape[1])
    prep.encode_latin1(t_list, lut, out=dev_b, width=b.shape[1])
    torch.cuda.synchronize()
    dev_s = time.perf_counter() - t0
    if not torch.equal(dev_a.cpu(), torch.from_numpy(a.view(np.int32))):
        raise SystemExit("device encoding differs from the bench codes")
    return {"pairs": B, "per_problem_s": per_problem * B, "per_problem_sample_pairs": n,
            "batch_host_s": host_s, "batch_device_s": dev_s,
            "speedup_host": per_problem * B / host_s, "speedup_device": per_problem * B / dev_s,
            "bytes_uploaded_device": int(ls.sum() + lt.sum()), "codes_bytes": int(a.nbytes + b.nbytes)}


# --------------------------------------------------------------------------- fwd + bwd

def fwd_bwd(torch, pairs, seed, steps=3):
    """The differentiation form: global Gotoh (open 0.5, extend 0.1) on cosine similarities
    of per-token embeddings (d = 128, lengths U[64, 256], BF16 product with FP32
    accumulation), forward vs forward + backward (path subgradient, embedding gradients
    through the product), and DTW (minimize, |x - y|) on Gaussian random walks (lengths
    U[128, 1024]) with gradients w.r.t. the series.  GCUPS over real cells."""
    from pyalign_gb300 import autograd as ag
    rng = np.random.default_rng(seed)
    g = torch.Generator(device="cuda").manual_seed(seed)
    ls = rng.integers(64, 257, pairs)
    lt = rng.integers(64, 257, pairs)
    lengths = np.stack([ls, lt], axis=1)
    cells = float((ls.astype(np.int64) * lt).sum())
    Es = torch.randn(pairs, 256, 128, device="cuda", generator=g)
    Et = torch.randn(pairs, 256, 128, device="cuda", generator=g)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    a = Es.clone().requires_grad_(True)
    b = Et.clone().requires_grad_(True)

    def run(backward):
        with torch.set_grad_enabled(backward):
            sc = ag.embedding_alignment_score(a, b, lengths, 0.5, 0.1, "global", "maximize")
        if backward:
            sc.sum().backward()
            a.grad = b.grad = None
        return sc

    for _ in range(2):
        run(True)
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(steps):
        run(False)
    ev[1].record()
    for _ in range(steps):
        run(True)
    ev[2].record()
    torch.cuda.synchronize()
    fwd = cells * steps / (ev[0].elapsed_time(ev[1]) / 1000) / 1e9
    fb = cells * steps / (ev[1].elapsed_time(ev[2]) / 1000) / 1e9

    # DTW on random walks
    nd = pairs
    dl = rng.integers(128, 1025, size=(nd, 2))
    dcells = float((dl[:, 0].astype(np.int64) * dl[:, 1]).sum())
    x0 = torch.cumsum(torch.randn(nd, 1024, device="cuda", generator=g), dim=1)
    y0 = torch.cumsum(torch.randn(nd, 1024, device="cuda", generator=g), dim=1)

    x = x0.clone().requires_grad_(True)
    y = y0.clone().requires_grad_(True)

    def run_dtw(backward):
        with torch.set_grad_enabled(backward):
            sc = ag.dtw_series_score(x, y, dl)
        if backward:
            sc.sum().backward()
            x.grad = y.grad = None
        return sc

    for _ in range(2):
        run_dtw(True)
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(steps):
        run_dtw(False)
    ev[1].record()
    for _ in range(steps):
        run_dtw(True)
    ev[2].record()
    torch.cuda.synchronize()
    dfwd = dcells * steps / (ev[0].elapsed_time(ev[1]) / 1000) / 1e9
    dfb = dcells * steps / (ev[1].elapsed_time(ev[2]) / 1000) / 1e9
    return {"value": fb, "unit": "GCUPS", "fwd_only": fwd, "fwd_bwd_over_fwd": fb / fwd,
            "workload": f"{pairs} pairs, global Gotoh 0.5/0.1 on cosine(E_s, E_t), d=128, L~U[64,256]",
            "dtw": {"fwd_bwd": dfb, "fwd_only": dfwd, "fwd_bwd_over_fwd": dfb / dfwd,
                    "workload": f"{nd} pairs, DTW |x-y| on Gaussian random walks, L~U[128,1024] "
                                "(series form: |x-y| computed in the DP kernel)"}}


def error_report(sc32, rep, scale, bound=1e-5):
    """Error of the float32 scores against the FP64 replay of each pair's recovered path:
    the largest error relative to |score|, how many pairs (and which fraction) exceed `bound`
    relative to |score| and the range of |score| among them, and -- where the magnitude of
    the summed terms is given (sum |S| over the aligned cells plus the gap costs) -- the
    largest error relative to it and how many pairs exceed `bound` that way."""
    err = (sc32.double() - rep).abs().cpu().numpy()
    mag = rep.abs().cpu().numpy()
    rel = err / np.maximum(mag, 1e-300)
    over = rel > bound
    out = {"pairs": int(len(rel)), "max_rel_score": float(rel.max()), "bound": bound,
           "over_bound_rel_score": int(over.sum()), "over_bound_fraction": float(over.mean()),
           "abs_score_of_those": [float(mag[over].min()), float(mag[over].max())] if over.any() else None,
           "median_abs_score": float(np.median(mag))}
    if scale is not None:
        rt = err / scale.cpu().numpy()
        out.update({"max_rel_terms": float(rt.max()), "over_bound_rel_terms": int((rt > bound).sum())})
        if over.any():
            out["score_over_terms_of_those_max"] = float((mag / scale.cpu().numpy())[over].max())
    return out


def precision_config(torch, pairs, seed, steps=3):
    """The precision form: global Gotoh (open 0.5, extend 0.1, maximize) on S = cos of
    per-token embeddings (d = 256, N(0, 1) then L2-normalised, lengths U[32, 512]) with the
    similarity product on the tensor cores (pa_similarity_bf16: BF16 factors, FP32
    accumulation in TMEM) and the float32 DP, plus the DTW variant (minimize) on 1 - cos
    written by the same kernel's epilogue.  Reports the product alone (TFLOP/s over the
    ragged cells' 2 d flops), the DP alone and normalise + product + DP (GCUPS over real
    cells), and the score error of the float32 DP against the FP64 replay of each pair's
    recovered path (pa_path_scores_f64), relative to |score| and to the summed terms."""
    from pyalign_gb300 import autograd as ag
    rng = np.random.default_rng(seed)
    g = torch.Generator(device="cuda").manual_seed(seed)
    n, d = 512, 256
    lengths = rng.integers(32, n + 1, size=(pairs, 2))
    ls, lt = lengths[:, 0].astype(np.int64), lengths[:, 1].astype(np.int64)
    cells = float((ls * lt).sum())
    Es = torch.randn(pairs, n, d, device="cuda", generator=g)
    Et = torch.randn(pairs, n, d, device="cuda", generator=g)
    St = torch.empty((pairs, n, n), dtype=torch.float32, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(8)]
    stream = torch.cuda.current_stream()

    def product(alpha=1.0, beta=0.0):
        # rows past each length: zero up to the product's tile, not read; not written beyond
        Esb, _ = ag.normalized_bf16(Es, True, ls, tiled=True)
        Etb, _ = ag.normalized_bf16(Et, True, lt, tiled=True)
        return ag.similarity_bf16(Esb, Etb, lengths, out=St, alpha=alpha, beta=beta), Esb, Etb

    S, Esb, Etb = product()
    ag._forward_paths(S, lengths, (0.5, 0.1), "global", "maximize", False)
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(steps):
        ag.similarity_bf16(Esb, Etb, lengths, out=St)
    ev[1].record(stream)
    for _ in range(steps):
        ag._forward_paths(S, lengths, (0.5, 0.1), "global", "maximize", False)
    ev[2].record(stream)
    for _ in range(steps):
        S, _, _ = product()
        ag._forward_paths(S, lengths, (0.5, 0.1), "global", "maximize", False)
    ev[3].record(stream)
    torch.cuda.synchronize()
    t_gemm = ev[0].elapsed_time(ev[1]) / 1000 / steps
    t_dp = ev[1].elapsed_time(ev[2]) / 1000 / steps
    t_all = ev[2].elapsed_time(ev[3]) / 1000 / steps
    # the float DP kernel alone (the solver's phase events of its last solve) against the
    # measured float32 add/add/max peak: global Gotoh 9 ops + one-optimal traceback 4 per cell
    dp_solver = ag._solver(pairs, n, n, "global", "maximize", False, (0.5, 0.1))
    ag._forward_paths(S, lengths, (0.5, 0.1), "global", "maximize", False)
    torch.cuda.synchronize()
    ms4, _ = dp_solver.last_timings()
    from pyalign_gb300 import algorithm as alg
    f32_peak, pms = ctypes.c_float(0), ctypes.c_float(0)
    alg.check(alg.lib().pa_measure_f32_peak(ctypes.byref(f32_peak), ctypes.byref(pms)))
    dp_kernel_s = ms4[1] / 1000.0
    f_ops = 13.0 * cells / dp_kernel_s / 1e9
    dp_roof = {"bound": "alu", "achieved": f_ops, "peak": float(f32_peak.value), "unit": "Gop/s",
               "frac": f_ops / float(f32_peak.value), "ops_per_cell": 13, "kernel_ms": ms4[1],
               "plan": dp_solver.last_plan(), "peak_source": "measured in-run (pa_measure_f32_peak)",
               "hbm": {"bytes_per_cell": 4.5, "achieved_gbs": 4.5 * cells / dp_kernel_s / 1e9,
                       "note": "S read (4 B) + traceback nibble (0.5 B) per cell"}}
    sc32, rep, scale = ag.path_scores_f64(S, lengths, 0.5, 0.1, "global", "maximize", with_scale=True)
    gotoh_err = error_report(sc32, rep, scale)

    D, _, _ = product(-1.0, 1.0)
    ag._forward_paths(D, lengths, None, "global", "minimize", True)
    torch.cuda.synchronize()
    ev[4].record(stream)
    for _ in range(steps):
        D, _, _ = product(-1.0, 1.0)
        ag._forward_paths(D, lengths, None, "global", "minimize", True)
    ev[5].record(stream)
    torch.cuda.synchronize()
    t_dtw = ev[4].elapsed_time(ev[5]) / 1000 / steps
    dsc, drep = ag.path_scores_f64(D, lengths, locality="global", direction="minimize", dtw=True)
    dtw_err = error_report(dsc, drep, None)
    status = ag.tensor_core_status()
    tiles = float((((lt + 127) // 128) * ((ls + 127) // 128)).sum())
    return {
        "value": cells / t_all / 1e9, "unit": "GCUPS",
        "workload": f"{pairs} pairs, L~U[32,{n}], d={d}, cos on the tensor cores, global Gotoh 0.5/0.1 (FP32 DP)",
        "product": {"ms": t_gemm * 1e3, "tflops": 2.0 * d * cells / t_gemm / 1e12,
                    "tile_tflops": 2.0 * d * tiles * 128 * 128 / t_gemm / 1e12,
                    "out_gbs": 4.0 * cells / t_gemm / 1e9, "status": status},
        "dp_gcups": cells / t_dp / 1e9, "dp_ms": t_dp * 1e3, "total_ms": t_all * 1e3,
        "dp_roofline": dp_roof,
        "error_vs_fp64_replay": gotoh_err,
        "dtw": {"value": cells / t_dtw / 1e9, "unit": "GCUPS", "ms": t_dtw * 1e3,
                "error_vs_fp64_replay": dtw_err,
                "workload": "DTW (minimize) on 1 - cos of the same pairs, distance from the product's epilogue"},
    }


# --------------------------------------------------------------------------- plain path

PLAIN_ENV = {"PA_TUNE": "0", "PA_GRAPHS": "0", "PA_GRID": "exact"}


def plain_gpu(torch, alg, L, a, b, ls, lt, t_d, stream, plan, width=100, steps=3):
    """The plain GPU path of the batched workload: the bag split into length buckets
    (|s| and |t| in 100-wide bins, each bucket padded to its own longest pair), one
    pa_solve_batch call (one DP launch and one walk launch, synchronised) per bucket, the
    plan fixed (no autotuner), no graph replay, a non-persistent grid (one warp per work
    unit).  Two kernels: the int32 one-column kernel at G = 8 (the analytic plan without the
    16-bit and two-column forms) and the kernel and G the batched form chose."""
    P = ctypes.POINTER
    lo = int(min(ls.min(), lt.min()))
    top = max(0, (int(max(ls.max(), lt.max())) - lo) // width - 1)   # the longest length joins the last bin
    key = np.minimum((ls - lo) // width, top) * 1000 + np.minimum((lt - lo) // width, top)
    buckets = []
    for kv in np.unique(key):
        idx = np.nonzero(key == kv)[0]
        n_s, n_t = int(ls[idx].max()), int(lt[idx].max())
        a_b = torch.from_numpy(np.ascontiguousarray(a[idx, :n_s]).view(np.int32)).cuda()
        b_b = torch.from_numpy(np.ascontiguousarray(b[idx, :n_t]).view(np.int32)).cuda()
        length = np.ascontiguousarray(np.stack([ls[idx], lt[idx]]), dtype=np.int32)
        sizes = np.minimum(ls[idx], lt[idx]).astype(np.int64)
        offs = np.zeros(len(idx), np.int64)
        offs[1:] = np.cumsum(sizes)[:-1]
        buckets.append(dict(n=len(idx), n_s=n_s, n_t=n_t, a=a_b, b=b_b, length=length, offs=offs,
                            sc=torch.empty(len(idx), dtype=torch.float32, device="cuda"),
                            mp=torch.empty(max(1, int(sizes.sum())), dtype=torch.int32, device="cuda")))
    cells = float((ls.astype(np.int64) * lt).sum())

    def run(env):
        saved = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        try:
            for bk in buckets:   # solvers and batch structs, outside the timed region
                mod = alg.m16
                bk["solver"] = mod.create_solver(bk["n_s"], bk["n_t"], mod.create_options(options_dict(alg, bk["n"])))
                alg.check(L.pa_solver_set_stream(bk["solver"].handle, ctypes.c_void_p(stream.cuda_stream)))
                bk["batch"] = alg.Batch(form=1, location=1, batch=bk["n"], n_s=bk["n_s"], n_t=bk["n_t"],
                                        a=ctypes.cast(bk["a"].data_ptr(), P(ctypes.c_uint32)),
                                        b=ctypes.cast(bk["b"].data_ptr(), P(ctypes.c_uint32)),
                                        table=ctypes.cast(t_d.data_ptr(), P(ctypes.c_float)), table_rows=4,
                                        table_cols=4, length=bk["length"].ctypes.data_as(P(ctypes.c_int32)))

            def one_pass():
                for bk in buckets:
                    alg.check(L.pa_solve_batch(bk["solver"].handle, ctypes.byref(bk["batch"]),
                                               ctypes.c_void_p(bk["sc"].data_ptr()), ctypes.c_void_p(bk["mp"].data_ptr()),
                                               bk["offs"].ctypes.data_as(P(ctypes.c_int64))))
            one_pass()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                one_pass()
            e1.record(stream)
            torch.cuda.synchronize()
            plans = {str(bk["solver"].last_plan()) for bk in buckets}
            return cells * steps / (e0.elapsed_time(e1) / 1000.0) / 1e9, sorted(plans)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    v_int32, plans_int32 = run(dict(PLAIN_ENV, PA_GROUP_WIDTH="8", PA_DP16="0", PA_DP_COLS="1"))
    same = dict(PLAIN_ENV, PA_GROUP_WIDTH=str(plan["G"]))
    if plan["arithmetic"] != "int16x2":
        same["PA_DP16"] = "0"
    v_same, plans_same = run(same)
    return {"value": v_int32, "unit": "GCUPS", "pairs": len(ls), "buckets": len(buckets),
            "bucket_width": width, "plans": plans_int32, "batched_over_plain": None,
            "workload": "the whole bag, one synchronous solve call per length bucket, device-resident codes",
            "same_kernel": {"value": v_same, "unit": "GCUPS", "plans": plans_same}}


# --------------------------------------------------------------------------- arms

def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    a, b, ls, lt, table = make_workload(args.pairs, args.seed)
    per_step = args.cpu_seconds / max(args.steps, 1)
    vals = []
    desc = None
    threads = os.cpu_count() or 1
    for k in range(args.warmup + args.steps):
        g, threads, desc, _, _, _ = cpu_baseline(a, b, ls, lt, table, per_step if k >= args.warmup else 1.0)
        if k >= args.warmup:
            vals.append(g)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "pairs": args.pairs, "sample_per_step": desc},
        "cpu_baseline": {"value": value, "unit": "GCUPS", "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of pyalign's solver.h (oracle/pa_oracle.cpp): the reference's xtensor "
                "core has no buildable sources here",
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from pyalign_gb300 import algorithm as alg
    from pyalign_gb300 import build as pbuild
    pbuild.build()
    L = alg.lib()
    L.pa_measure_int32_peak.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    L.pa_measure_int16x2_peak.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    L.pa_solver_last_bytes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]

    # each rank solves its own batch (pairs are independent: weak scaling, no collective)
    a, b, ls, lt, table = make_workload(args.pairs, args.seed + rank)
    B = args.pairs
    cells = int((ls.astype(np.int64) * lt.astype(np.int64)).sum())
    mod = alg.m16
    solver = mod.create_solver(1000, 1000, mod.create_options(options_dict(alg, B)))
    stream = torch.cuda.current_stream()
    alg.check(L.pa_solver_set_stream(solver.handle, ctypes.c_void_p(stream.cuda_stream)))

    length = np.ascontiguousarray(np.stack([ls, lt]), dtype=np.int32)
    sizes = np.minimum(ls, lt).astype(np.int64)
    offs = np.zeros(B, np.int64)
    offs[1:] = np.cumsum(sizes)[:-1]
    nmap = int(sizes.sum())

    # device-resident inputs and outputs
    a_d = torch.from_numpy(a.view(np.int32)).cuda()
    b_d = torch.from_numpy(b.view(np.int32)).cuda()
    t_d = torch.from_numpy(table).cuda()
    sc_d = torch.empty(B, dtype=torch.float32, device="cuda")
    mp_d = torch.empty(nmap, dtype=torch.int32, device="cuda")

    def batch_struct(loc, aa, bb, tt):
        P = ctypes.POINTER
        return alg.Batch(form=1, location=loc, batch=B, n_s=a.shape[1], n_t=b.shape[1],
                         a=ctypes.cast(aa, P(ctypes.c_uint32)), b=ctypes.cast(bb, P(ctypes.c_uint32)),
                         table=ctypes.cast(tt, P(ctypes.c_float)), table_rows=4, table_cols=4,
                         length=length.ctypes.data_as(P(ctypes.c_int32)))

    dev_batch = batch_struct(1, a_d.data_ptr(), b_d.data_ptr(), t_d.data_ptr())
    offs_p = offs.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))

    def step_device():
        alg.check(L.pa_solve_batch(solver.handle, ctypes.byref(dev_batch), ctypes.c_void_p(sc_d.data_ptr()),
                                   ctypes.c_void_p(mp_d.data_ptr()), offs_p))

    # pinned host buffers for the end-to-end form
    a_h = torch.from_numpy(a.view(np.int32)).pin_memory()
    b_h = torch.from_numpy(b.view(np.int32)).pin_memory()
    t_h = torch.from_numpy(table).pin_memory()
    sc_h = torch.empty(B, dtype=torch.float32).pin_memory()
    mp_h = torch.empty(nmap, dtype=torch.int32).pin_memory()
    host_batch = batch_struct(0, a_h.data_ptr(), b_h.data_ptr(), t_h.data_ptr())

    def step_host():
        alg.check(L.pa_solve_batch(solver.handle, ctypes.byref(host_batch), ctypes.c_void_p(sc_h.data_ptr()),
                                   ctypes.c_void_p(mp_h.data_ptr()), offs_p))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---- device-resident timing
    clocks = ClockSampler(local).start()
    for _ in range(args.warmup):
        step_device()
    barrier()
    dp_ms, walk_ms, up_ms, down_ms, launches = [], [], [], [], 0
    ms4 = (ctypes.c_float * 4)()
    nl = ctypes.c_int32(0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.begin("device")
    e0.record(stream)
    for _ in range(args.steps):
        step_device()
        L.pa_solver_last_timings(solver.handle, ms4, ctypes.byref(nl))
        up_ms.append(ms4[0])
        dp_ms.append(ms4[1])
        walk_ms.append(ms4[2])
        down_ms.append(ms4[3])
        launches += nl.value
    e1.record(stream)
    barrier()
    clocks.end("device")
    elapsed = max_over_ranks(e0.elapsed_time(e1) / 1000.0)
    value = cells * world * args.steps / elapsed / 1e9
    plan = solver.last_plan()

    # correctness spot check of the device results against the host path below
    sc_dev = sc_d.cpu().numpy().copy()

    # ---- end-to-end timing through the C ABI with host buffers
    for _ in range(max(1, args.warmup)):
        step_host()
    barrier()
    clocks.begin("e2e")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    clocks.end("e2e")
    clocks.stop()
    e2e = cells * world * args.steps / e2e_s / 1e9
    h2d, d2h = ctypes.c_int64(0), ctypes.c_int64(0)
    L.pa_solver_last_bytes(solver.handle, ctypes.byref(h2d), ctypes.byref(d2h))
    if not np.array_equal(sc_dev, sc_h.numpy()):
        raise SystemExit("device-resident and host-buffer runs disagree")

    # ---- the reference-facing module call: Solver.solve_indexed_for_alignment, the native
    # method pyalign's indexed form calls for a batch (solve.py:399-432), with host numpy
    # arrays in the layouts pyalign builds (codes uint32 (batch, n), lengths uint16 (2, batch))
    # and its result as a tuple of Alignment objects
    ln16 = np.stack([ls, lt]).astype(np.uint16)
    api_solver = mod.create_solver(1000, 1000, mod.create_options(options_dict(alg, B)))
    alg.check(L.pa_solver_set_stream(api_solver.handle, ctypes.c_void_p(stream.cuda_stream)))
    for _ in range(max(2, args.warmup)):  # the first call plans, the first repeat sets up its pipeline
        api_res = api_solver.solve_indexed_for_alignment(a, b, table, ln16)
    barrier()
    api_steps = max(3, args.steps // 4)
    api_calls = []
    t0 = time.perf_counter()
    for _ in range(api_steps):
        t1 = time.perf_counter()
        api_res = api_solver.solve_indexed_for_alignment(a, b, table, ln16)
        api_calls.append((time.perf_counter() - t1) * 1000)
    barrier()
    api_s = max_over_ranks(time.perf_counter() - t0)
    L.pa_solver_last_timings(api_solver.handle, ms4, ctypes.byref(nl))
    api_phases = {"upload": ms4[0], "dp": ms4[1], "traceback": ms4[2], "download": ms4[3]}
    if float(api_res[0].score) != float(sc_h[0]) or not np.array_equal(
            np.asarray(api_res[B - 1].s_to_t if ls[B - 1] <= lt[B - 1] else api_res[B - 1].t_to_s),
            mp_h.numpy()[offs[B - 1]:offs[B - 1] + sizes[B - 1]]):
        raise SystemExit("module call and pa_solve_batch disagree")
    t0 = time.perf_counter()
    n_obj = sum(1 for _ in api_res)
    objects_ms = (time.perf_counter() - t0) * 1000
    e2e_api = {"value": cells * world * api_steps / api_s / 1e9, "unit": "GCUPS", "steps": api_steps,
               "call": "Solver.solve_indexed_for_alignment of the native module (one call for the whole bag), "
                       "host numpy arrays; returns the per-lane sequence of Alignment objects, each made at its "
                       "first access",
               "call_ms": api_calls, "phases_ms_last_call": api_phases,
               "objects_ms": objects_ms, "objects": n_obj,
               "objects_note": "making all Alignment objects of one call by iterating the sequence (outside the "
                               "timed calls; pyalign's own loop does this, solve.py:374-379)"}
    del api_res

    # ---- the plain GPU path: one launch per length bucket (100-wide bins of |s| and |t|)
    # over the whole bag, device-resident codes, one synchronous solve call per bucket, fixed
    # plan (no tuner), no graphs, a non-persistent grid; "plain" runs the int32 one-column
    # kernel at G = 8, "plain_same_kernel" the batched form's kernel and width per bucket
    # (measured after the end-to-end runs: its many short-lived solvers are not in their way)
    plain = None
    if args.plain:
        plain = plain_gpu(torch, alg, L, a, b, ls, lt, t_d, stream, plan)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # ---- roofline of the DP kernel (integer ALU bound; traceback stores are the HBM side).
    # The denominator is the measured peak of the arithmetic the chosen kernel computes in:
    # int32 lanes, or packed 16-bit pairs (two lane operations per instruction).
    packed = plan["arithmetic"] == "int16x2"
    peak32, peak16 = ctypes.c_float(0), ctypes.c_float(0)
    pms = ctypes.c_float(0)
    alg.check(L.pa_measure_int32_peak(ctypes.byref(peak32), ctypes.byref(pms)))
    alg.check(L.pa_measure_int16x2_peak(ctypes.byref(peak16), ctypes.byref(pms)))
    peak = peak16 if packed else peak32
    peak_fn = "pa_measure_int16x2_peak" if packed else "pa_measure_int32_peak"
    dp_s = statistics.mean(dp_ms) / 1000.0
    achieved_ops = cells * OPS_PER_CELL / dp_s / 1e9
    peaks = {}
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    alg_bytes = cells * BYTES_PER_CELL + float((ls.astype(np.int64) + lt.astype(np.int64)).sum()) * 4
    traffic = None
    prof = os.path.join(REPO, "profiles", "dp16_affine_local_traffic.json" if packed else "dp_affine_local_traffic.json")
    if os.path.exists(prof):
        with open(prof) as f:
            pj = json.load(f)
        traffic = pj["dram_bytes_per_cell"] * cells
    roof_alu = {"bound": "alu", "achieved": achieved_ops, "peak": float(peak.value), "unit": "Gop/s",
                "frac": achieved_ops / float(peak.value), "traffic": traffic,
                "ops_per_cell": OPS_PER_CELL, "peak_source": f"measured in-run ({peak_fn})",
                "int32_peak": float(peak32.value), "int16x2_peak": float(peak16.value)}
    roof_hbm = {"bound": "hbm", "achieved": alg_bytes / dp_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": alg_bytes / dp_s / 1e9 / hbm_peak, "traffic": traffic,
                "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "of fallback"}

    fb = fwd_bwd(torch, args.fwd_bwd_pairs, args.seed + 5) if args.fwd_bwd_pairs > 0 else None
    others = other_configs(torch, alg, L, args.seed + 7, args.allopt_pairs) if args.other_configs else None
    prec = precision_config(torch, args.precision_pairs, args.seed + 2) if args.precision_pairs > 0 else None
    prepd = prepare_config(torch, a, b, ls, lt) if args.prepare else None

    # CPU baseline on all host threads and on one core; the oracle's scores and alignment
    # maps of the sampled pairs are compared bit for bit with the GPU arm's (exit 1 on any
    # difference, after the line is printed)
    cpu, parity = None, None
    if not args.no_cpu_baseline and world == 1:
        g, threads, desc, n_par, sc_ref, mp_ref = cpu_baseline(a, b, ls, lt, table, args.cpu_seconds)
        g1, _, desc1, _, _, _ = cpu_baseline(a, b, ls, lt, table, args.cpu_seconds / 2, threads=1)
        cpu = {"value": g, "unit": "GCUPS", "cores": threads, "kind": "port", "sample": desc,
               "one_core": {"value": g1, "unit": "GCUPS", "cores": 1, "sample": desc1}}
        parity = dict(parity_of(n_par, sc_ref, mp_ref, sc_h.numpy(), mp_h.numpy()),
                      against="oracle (CPU restatement of the reference's solver)",
                      arm="e2e (host buffers); the device-resident run's scores equal it")

    if plain is not None:
        plain["batched_over_plain"] = value / plain["value"]
        plain["same_kernel"]["batched_over_plain_same_kernel"] = value / plain["same_kernel"]["value"]
    line = {
        "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed * 1000.0 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16x2" if packed else "int32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "pairs": B, "cells_per_step": cells, "form": "indexed (a, b uint32 codes)",
                   "l2": "inputs larger than L2: 524 MB of codes and ~14 GB of traceback masks per step",
                   "parallelism": f"dp{world} (independent pairs per GPU)"},
        "parity": parity,
        "roofline": roof_alu,
        "roofline_hbm": roof_hbm,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": "GCUPS", "h2d_bytes_per_step": int(h2d.value),
                "d2h_bytes_per_step": int(d2h.value)},
        "e2e_api": e2e_api,
        "gpu_launches": launches,
        "plain_gpu": plain,
        "fwd_bwd": fb,
        "other_configs": others,
        "precision": prec,
        "prepare": prepd,
        "kernel_ms_per_step": {"dp": statistics.mean(dp_ms), "traceback": statistics.mean(walk_ms),
                               "before_dp": statistics.mean(up_ms), "after_traceback": statistics.mean(down_ms)},
        "plan": plan,
        "clocks": dict(clocks.summary("device"), e2e=clocks.summary("e2e")),
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    bad = [k for k, v in (("bench", parity), *((k, v.get("parity")) for k, v in (others or {}).items()))
           if v is not None and v["mismatches"]]
    bad += [k for k, v in (others or {}).items() if v.get("same_results") is False]
    if bad:
        print(f"parity failure against the oracle: {bad}", file=sys.stderr)
        sys.exit(1)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

#!/usr/bin/env python3
"""Benchmark of the sparse upper-triangular solve on the large irregular single-RHS system.

Workload (one "step" = one complete solve of U x = b to relative residual <= 1e-12):
  n = 2,000,000 upper-triangular CSR; per row Poisson(8) off-diagonals, each at i + U{1..64}
  with probability 0.9 else U{i+1..n-1}; values U[-1,1]; diagonal 1 + sum |off|; FP64;
  b = U x*, x* ~ U[-1,1]; seed 1 (sptrsv_gb300/gen.py).  Seeded synthetic data.

Reported (one JSON line on rank 0):
  value        solves/s of the chosen form (FP32 bulk solve + FP64 iterative refinement,
               schedule from the matrix features), inputs resident in HBM, device time of
               each step with CUDA events on the solver's stream, L2 flushed between steps;
  e2e          the same through the public C ABI with pinned host b / x: every step copies b
               to the device and brings x back inside its timed region (x is written to the
               pinned host buffer by the FP64 residual kernels over the C2C link, the converged
               one last, so no copy follows the solve);
  plain_fp64_syncfree  the plain FP64 sync-free GPU solve on the same system (the baseline the
               chosen form is compared with);
  fp64_refined the same refinement run to FP64 accuracy (relative residual 1e-15), the form the
               drop-in base_gauss_upper takes on this system;
  roofline     the dominant kernel of the chosen form: its algorithmic bytes per launch over
               its average launch time (CUDA events between kernels, same steps), against the
               measured HBM copy bandwidth;
  cpu_baseline the reference's CPU paths (serial backward substitution, OpenMP level-set on
               all host cores) timed on this host, best of the two.
--impl reference runs the reference's CPU implementation (oracle/_ref when it was compiled
from the reference sources on this host, else the oracle's C restatement) as the arm of
comparison.  Multi-GPU: replicas (one system per rank, no collective); value sums all ranks.

Other workloads (their own JSON line, same keys where they apply):
  --workload batch       the batched uneven mix: 512 systems, n log-uniform in [1k, 200k], half
                         banded 2D-Laplacian Cholesky factors, half random dominant factors, RHS
                         1-16, seed 2.  value = systems solved per second by the per-system
                         schedules the trained selector picks (one CUDA graph, device-driven
                         refinement); plain_fp64_syncfree = every system by the FP64 pull in one
                         persistent launch; per-kernel device times from an event-timed replay.
  --workload supernodal  the 40^3 nested-dissection factor at 1, 8, 32 and 128 right-hand sides:
                         FP64 supernodal, BF16x3 supernodal + FP64 refinement, plain FP64
                         sync-free, serial CPU.
  --workload dropin      the reference-signature base_gauss_upper on the 64 x 64 and 256 x 256
                         grid Laplacian factors and the 2M-row system, against the serial CPU solve.
  --workload factor      the step upstream of the supernodal solve: the GPU multifrontal Cholesky
                         of the 40^3 nested-dissection 3D Laplacian (sptrsv_factor_multifrontal),
                         beside the host generator's numpy/scipy factor of the same fronts.
"""
import argparse
import csv
import io
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

METRIC = "solves/sec & HBM GB/s: chosen vs plain FP64 sync-free, at rel. resid <=1e-12"
WORKLOAD = ("irregular-2M: n=2,000,000 upper CSR, Poisson(8) off-diagonals/row, 90% at offset U{1..64}, "
            "10% uniform to the right, FP64, diag=1+sum|off|, b=U x*, seed 1, single RHS")
RES_TOL = 1e-12
# the plain FP64 sync-free baseline of the single-system workload: the fastest exact sync-free
# kernel for one RHS
PLAIN_SCHEDULE = "syncfree_window"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=2_000_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="irregular2m",
                    choices=["irregular2m", "batch", "supernodal", "dropin", "factor"],
                    help="irregular2m: the 2M-row single solve (default); batch: the 512-system uneven mix; "
                         "supernodal: the 40^3 nested-dissection factor at 1/8/32/128 right-hand sides; "
                         "dropin: the reference-signature base_gauss_upper on three systems; "
                         "factor: the GPU multifrontal Cholesky that produces the supernodal factor")
    ap.add_argument("--grid", type=int, default=40, help="factor: side of the 3D Laplacian grid")
    ap.add_argument("--count", type=int, default=512, help="batch: number of systems")
    ap.add_argument("--nmax", type=int, default=200_000, help="batch: largest n")
    ap.add_argument("--batch-steps", type=int, default=10,
                    help="default workload: timed steps of the batched mix measured after the 2M-row system")
    ap.add_argument("--no-batch", action="store_true", help="default workload: skip the nested batched-mix record")
    ap.add_argument("--panels", default="fp64", choices=["fp64", "tc", "df"],
                    help="panel products of the exact FP64 supernodal / batched schedules: FP64 FMAs, the tensor "
                         "cores (BF16 digit slices) or double-FP32 on the FP32 pipes; all FP64-accurate")
    ap.add_argument("--rhs", default="1,8,32,128", help="supernodal: right-hand-side counts (comma list)")
    ap.add_argument("--plain-schedule", default=None, choices=["syncfree_block", "syncfree_window", "syncfree_warp"],
                    help="default workload: the plain FP64 sync-free baseline's schedule")
    return ap.parse_args()


# ---------------------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.ws = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        """Starts sampling every 50 ms and returns once the first sample is written (at most 5 s),
        so that the timed region that follows is covered from its start."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        t0 = time.time()
        while time.time() - t0 < 5.0 and self.proc.poll() is None:
            self.f.flush()
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.f.read())) if len(r) >= 9]
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(kernel):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, when one exists."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    try:
        for line in open(p):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel:
                return float(parts[1])
    except OSError:
        pass
    return None


def fp64_bytes(n, nnz, rhs=1):
    """Algorithmic bytes of one FP64 solve: every entry (value + column index) once, the row
    pointer once, B read and X written once (x gathers assumed cache-resident)."""
    return 12 * nnz + 4 * (n + 1) + 16 * n * rhs


def jacobi_bytes(n, nnz):
    """Algorithmic bytes of one FP32 Jacobi sweep: off-diagonal values + columns (8 B each),
    row pointer, FP32 reciprocal diagonal, r, the previous iterate (read once) and the new
    iterate (written once)."""
    return 8 * (nnz - n) + 4 * (n + 1) + 4 * n * 4


# ---------------------------------------------------------------------------------------
def cpu_model():
    """The host CPU as /proc/cpuinfo names it (model name, or implementer/part on Arm)."""
    try:
        info = open("/proc/cpuinfo").read()
        for key in ("model name", "Model"):
            for line in info.splitlines():
                if line.startswith(key):
                    return line.split(":", 1)[1].strip()
        impl = [l.split(":")[1].strip() for l in info.splitlines() if l.startswith("CPU implementer")]
        part = [l.split(":")[1].strip() for l in info.splitlines() if l.startswith("CPU part")]
        if impl and part:
            return f"{os.uname().machine} implementer {impl[0]} part {part[0]}"
    except OSError:
        pass
    return os.uname().machine


def cpu_paths(m, b, budget_s=8.0):
    """Times the reference's CPU paths on this host; returns a dict with the best."""
    from oracle import oracle
    R = oracle.ref()
    kind = "reference" if R is not None else "port"
    rpu = m.row_ptr.astype(np.uint64)
    cores = os.cpu_count() or 1
    x = np.zeros(m.n)
    res = {}

    def serial():
        if R is not None:
            R.ref_base_gauss_upper(m.n, m.val, rpu, m.col, x, b, 1)
        else:
            oracle.lib().orc_base_gauss_upper(m.n, m.val, rpu, m.col, x, b, 1)

    def levelset():
        if R is not None:
            R.ref_barrier_upper(m.n, x, b, m.val, m.col, rpu, cores, 1)
        else:
            oracle.barrier_upper(rpu, m.col, m.val, b, 1, num_threads=cores)

    def levelset1():
        if R is not None:
            R.ref_barrier_upper(m.n, x, b, m.val, m.col, rpu, 1, 1)
        else:
            oracle.barrier_upper(rpu, m.col, m.val, b, 1, num_threads=1)

    for name, fn, threads in (("serial base_gauss_upper", serial, 1), ("level-set barrier_upper", levelset, cores),
                              ("level-set barrier_upper, 1 thread", levelset1, 1)):
        fn()
        t0 = time.perf_counter()
        reps = 0
        while True:
            fn()
            reps += 1
            el = time.perf_counter() - t0
            if reps >= 2 and el >= budget_s / 2 or reps >= 50 or el >= budget_s:
                break
        res[name] = {"solves_per_s": reps / el, "threads": threads, "reps": reps}
    best = max(res, key=lambda k: res[k]["solves_per_s"])
    return {"value": res[best]["solves_per_s"], "unit": "solves/s", "cores": res[best]["threads"], "kind": kind,
            "sample": f"{best} on the full system, {res[best]['reps']} solves timed on the host "
                      f"({cpu_model()}, {cores} cores); other paths: "
                      + "; ".join(f"{k} {v['solves_per_s']:.3g} solves/s ({v['threads']} thr)" for k, v in res.items()
                                  if k != best),
            "paths": res, "best": best, "fn": serial if best.startswith("serial") else levelset}


def errors_vs_serial(m, b, solutions):
    """Error of each GPU solution against the reference's serial FP64 solve of the same system
    (the oracle's C restatement, whose outputs the golden tests pin to the compiled reference):
    relative residual
    ||b - U x|| / ||b|| and max_i |x_i - x_ref_i| / |x_ref_i| (components with |x_ref_i| < 1e-12
    are measured against 1e-12), plus the reference-style relative 2-norm error (utils.cpp:355-380)."""
    from oracle import oracle
    rpu = m.row_ptr.astype(np.uint64)
    x_ref = oracle.base_gauss_upper(rpu, m.col, m.val, b, 1)
    out = {"oracle": "serial base_gauss_upper (core.cpp:18-32), FP64"}
    for name, xg in solutions.items():
        out[name] = {"rel_residual": oracle.rel_residual(rpu, m.col, m.val, xg, b, 1),
                     "max_elem_rel_error": oracle.max_elem_rel_error(x_ref, xg, 1e-12),
                     "rel_error_2norm": oracle.rel_error(x_ref, xg)}
    return out


def run_reference_batch(args):
    """The reference's serial solve over the batched mix: each step solves a bounded random
    sample of the systems (10 s, less when there are more than 12 steps, so that the run stays
    near two minutes) and is projected to the whole mix by nnz x rhs."""
    from sptrsv_gb300 import gen
    M = gen.mix(count=args.count, seed=2, nmin=1000, nmax=args.nmax)
    for k in range(args.warmup):
        batch_cpu_sample(M, budget_s=2.0, seed=100 + k)
    vals, t_all = [], time.perf_counter()
    cb = None
    budget = min(10.0, max(0.5, 120.0 / max(1, args.steps)))  # the whole run stays near two minutes
    for k in range(args.steps):
        cb = batch_cpu_sample(M, budget_s=budget, seed=k)
        vals.append(cb["value"])
    el = time.perf_counter() - t_all
    v = float(len(vals) / np.sum(1.0 / np.array(vals)))  # harmonic mean of the projected rates
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * args.count / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": BATCH_WORKLOAD.format(count=args.count, nmax=args.nmax), "systems": args.count},
            "cpu_baseline": cb, "wall_s": el,
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    M.close()


def run_reference(args, dist):
    if dist.rank != 0:
        return
    if args.workload == "batch":
        return run_reference_batch(args)
    from sptrsv_gb300 import gen
    from oracle import oracle
    oracle.build()
    m, xs, b = gen.irregular_case(args.n)
    cb = cpu_paths(m, b, budget_s=4.0)
    fn = cb.pop("fn")
    for _ in range(args.warmup):
        fn()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fn()
    el = time.perf_counter() - t0
    v = args.steps / el
    cb.pop("paths")
    cb.pop("best")
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n": m.n, "nnz": m.nnz, "rhs": 1},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------
def run_ours(args, dist):
    import sptrsv_gb300 as sp
    from sptrsv_gb300 import gen
    L = sp._lib.lib()
    m, xs, b = gen.irregular_case(args.n)
    s = sp.Solver(dist.local)
    s.analyse(m.row_ptr, m.col, m.val)
    info = s.info()
    n, nnz = m.n, m.nnz
    h = s.handle
    nbytes = 8 * n
    d_b, d_x = __import__("ctypes").c_void_p(), __import__("ctypes").c_void_p()
    import ctypes
    assert L.sptrsv_device_alloc(h, nbytes, ctypes.byref(d_b)) == 0
    assert L.sptrsv_device_alloc(h, nbytes, ctypes.byref(d_x)) == 0
    L.sptrsv_copy_h2d(h, d_b, b.ctypes.data, nbytes)
    assert s.sync() == 0

    chosen = sp.make_opts(precision="mixed", schedule="auto")
    plain = sp.make_opts(schedule=PLAIN_SCHEDULE)
    fp64r = sp.make_opts(schedule="jacobi")  # FP64 accuracy through refinement (residual 1e-15)

    def dev_solve(o):
        rc = L.sptrsv_solve(h, ctypes.byref(o), d_b, d_x, 1, sp.COL_MAJOR)
        if rc:
            raise sp.SptrsvError(rc, "solve")

    def timed_steps(o, steps, flush=True):
        ms = []
        fms = ctypes.c_float()
        for _ in range(steps):
            if flush:
                L.sptrsv_flush_l2(h)
            L.sptrsv_timer_begin(h)
            dev_solve(o)
            L.sptrsv_timer_end(h, ctypes.byref(fms))
            ms.append(fms.value)
            rc = s.sync()  # outside the events: reads the status and the device-looped launch count
            if rc:
                raise sp.SptrsvError(rc, "timed solve")
        return ms

    # correctness of both forms before timing
    x = np.empty(n)
    x_plain = np.empty(n)
    x_fp64r = np.empty(n)
    dev_solve(fp64r)
    if s.sync():
        raise SystemExit("FP64 refinement form did not converge")
    fp64r_res = s.last_refine()[1]
    L.sptrsv_copy_d2h(h, x_fp64r.ctypes.data, d_x, nbytes)
    for o in (chosen, plain):
        dev_solve(o)
        rc = s.sync()
        if rc:
            raise sp.SptrsvError(rc, "check solve")
    L.sptrsv_copy_d2h(h, x_plain.ctypes.data, d_x, nbytes)
    dev_solve(chosen)
    assert s.sync() == 0
    steps_ref, rel_res = s.last_refine()
    sweeps_ref = s.last_sweeps()
    L.sptrsv_copy_d2h(h, x.ctypes.data, d_x, nbytes)
    assert s.sync() == 0
    err_xstar = float(np.max(np.abs(x - xs)))
    if not rel_res <= RES_TOL:
        raise SystemExit(f"chosen form missed the tolerance: {rel_res}")

    # warm-up + timed region (chosen form)
    timed_steps(chosen, args.warmup)
    clocks = Clocks(dist.local)
    clocks.start()
    dist.barrier()
    assert s.sync() == 0
    l0 = s.launches()
    ms = timed_steps(chosen, args.steps)
    l1 = s.launches()
    ck = clocks.stop()
    dist.barrier()
    total_s = dist.max(sum(ms) / 1e3)
    value = dist.ws * args.steps / total_s
    gpu_launches = l1 - l0

    # plain FP64 sync-free on the same system
    psteps = max(3, min(args.steps, 5))
    timed_steps(plain, 1)
    pms = timed_steps(plain, psteps)
    plain_sps = psteps / (sum(pms) / 1e3)
    rsteps = max(3, min(args.steps, 20))
    timed_steps(fp64r, 1)
    rms = timed_steps(fp64r, rsteps)
    fp64r_sps = rsteps / (sum(rms) / 1e3)

    # per-kernel times of the chosen form: CUDA events between kernels, on an unlooped replay of
    # the same work (the corrections and sweeps per correction the device loop chose above)
    prof_opts = sp.make_opts(precision="mixed", schedule="auto", max_refine=max(1, steps_ref),
                             inner_sweeps=max(2, round(sweeps_ref / max(1, steps_ref))))
    s.profile(True)
    dev_solve(prof_opts)
    s.sync()
    per_kind = {}
    prof_steps = max(3, min(args.steps, 10))
    for _ in range(prof_steps):
        L.sptrsv_flush_l2(h)
        dev_solve(prof_opts)
        for kind, t in s.profile_read():
            per_kind.setdefault(kind, []).append(t)
    s.profile(False)
    kind_names = {1: "fill", 2: "pull_warp", 3: "pull_thread", 4: "push_csc", 5: "levelset", 6: "init",
                  7: "residual", 8: "check", 9: "jacobi_sweep", 10: "inner_exact", 11: "axpy", 12: "transpose"}
    shares = {kind_names.get(k, str(k)): {"launches_per_solve": len(v) / prof_steps, "total_ms_per_solve": sum(v) / prof_steps}
              for k, v in per_kind.items()}
    dom_kind = max(per_kind, key=lambda k: sum(per_kind[k]))
    dom_times = [t for t in per_kind[dom_kind] if t > 0]
    dom_avg_ms = sum(dom_times) / len(dom_times)
    if dom_kind == 9:
        dom_bytes, dom_name = jacobi_bytes(n, nnz), "k_jacobi_pairs"
    elif dom_kind == 7:
        dom_bytes, dom_name = fp64_bytes(n, nnz) - 8 * n, "k_residual_tile"
    else:
        dom_bytes, dom_name = fp64_bytes(n, nnz), kind_names.get(dom_kind, str(dom_kind))
    peak, peak_src = measured_peak()
    achieved = dom_bytes / (dom_avg_ms * 1e-3) / 1e9
    traffic = profiled_traffic(dom_name)

    # e2e through the C ABI with pinned host buffers
    hb, hx = ctypes.c_void_p(), ctypes.c_void_p()
    assert L.sptrsv_host_alloc(h, nbytes, ctypes.byref(hb)) == 0
    assert L.sptrsv_host_alloc(h, nbytes, ctypes.byref(hx)) == 0
    ctypes.memmove(hb, b.ctypes.data, nbytes)
    e2e_ms = []
    fms = ctypes.c_float()
    for k in range(args.warmup + args.steps):
        L.sptrsv_flush_l2(h)
        L.sptrsv_timer_begin(h)
        rc = L.sptrsv_solve_host(h, ctypes.byref(chosen), hb, hx, 1, sp.COL_MAJOR)
        L.sptrsv_timer_end(h, ctypes.byref(fms))
        if rc:
            raise sp.SptrsvError(rc, "e2e solve")
        if k >= args.warmup:
            e2e_ms.append(fms.value)
    xe = np.ctypeslib.as_array(ctypes.cast(hx, ctypes.POINTER(ctypes.c_double)), shape=(n,)).copy()
    assert np.max(np.abs(xe - xs)) <= 1e-8
    e2e_total = dist.max(sum(e2e_ms) / 1e3)
    e2e_value = dist.ws * args.steps / e2e_total

    cpu = None
    vs_oracle = None
    if dist.rank == 0 and dist.ws >= 1 and not args.no_cpu_baseline:
        try:
            cb = cpu_paths(m, b)
            cb.pop("fn")
            cb.pop("paths")
            cb.pop("best")
            cpu = cb
            vs_oracle = errors_vs_serial(m, b, {"chosen": x, "plain_fp64_syncfree": x_plain,
                                                "fp64_refined": x_fp64r})
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "solves/s", "error": str(e)[:200]}

    L.sptrsv_host_free(h, hb)
    L.sptrsv_host_free(h, hx)
    L.sptrsv_device_free(h, d_b)
    L.sptrsv_device_free(h, d_x)

    if dist.rank != 0:
        s.close()
        if not args.no_batch:
            batch_record(args, dist, max(1, args.batch_steps), max(3, min(args.warmup, 5)), with_cpu=False)
        return
    ms_step = 1e3 * total_s / args.steps
    fb = fp64_bytes(n, nnz)
    pipe = fp64_pipe(dist.local)
    sm_mhz = (ck or {}).get("sm_mhz") or 2070.0
    levels = int(info["max_level"])
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": dist.ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": n, "nnz": nnz, "max_level": info["max_level"], "rhs": 1,
                   "form": "FP32 Jacobi inner sweeps + FP64 residual/update (iterative refinement), one CUDA "
                           "graph with device-driven WHILE loops",
                   "l2": "512 MiB L2 flush between timed steps (outside the events); matrix 206 MB > L2",
                   "parallelism": f"replicas x{dist.ws}"},
        "hbm_gbs": fb * value / dist.ws / 1e9,
        "hbm_frac": fb * value / dist.ws / 1e9 / peak,
        "us_per_solve": 1e6 / (value / dist.ws),
        "gflops": (2 * (nnz - n) + n) * value / 1e9,
        "rel_residual": rel_res, "refine_steps": steps_ref, "inner_sweeps": sweeps_ref,
        "max_abs_err_vs_xstar": err_xstar,
        "vs_oracle": vs_oracle,
        "plain_fp64_syncfree": {"solves_per_s": plain_sps, "ms_per_solve": 1e3 / plain_sps,
                                "hbm_gbs": fb * plain_sps / 1e9, "schedule": PLAIN_SCHEDULE,
                                "ns_per_level": 1e9 / plain_sps / levels},
        "speedup_vs_plain": value / dist.ws / plain_sps,
        # the single-solve target of >= 40 % of the HBM-bytes roofline, stated over the whole solve
        # (one FP64 solve's algorithmic bytes per chosen-form solve), and the exact solve's
        # critical-path bound: one dependent FP64 FMA per level
        "single_solve_roofline": {"hbm_frac_whole_solve": fb * value / dist.ws / 1e9 / peak, "target": 0.40,
                                  "met": fb * value / dist.ws / 1e9 / peak >= 0.40,
                                  "dominant_kernel_frac": achieved / peak},
        "critical_path": {"levels": levels, "dep_fma_cycles": pipe["dep_fma_cycles"], "sm_mhz": sm_mhz,
                          "bound_ms_one_fma_per_level": levels * pipe["dep_fma_cycles"] / (sm_mhz * 1e3),
                          "plain_ms": 1e3 / plain_sps, "fp64_pipe_gfma_per_s": pipe["gfma_per_s"]},
        "fp64_refined": {"solves_per_s": fp64r_sps, "ms_per_solve": 1e3 / fp64r_sps, "rel_residual": fp64r_res,
                         "form": "FP64 accuracy through refinement: FP32 Jacobi sweeps, FP64 residuals to 1e-15"},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic,
                     "algorithmic_bytes_per_launch": dom_bytes, "avg_launch_ms": dom_avg_ms},
        "kernel_shares": shares,
        "gpu_launches": gpu_launches,
        "clocks": ck,
        "cpu_baseline": cpu,
    }
    s.close()
    if not args.no_batch:
        # the batched mix (the configuration of the >= 2x chosen-vs-plain target), same run
        rec = batch_record(args, dist, max(1, args.batch_steps), max(3, min(args.warmup, 5)),
                           with_cpu=not args.no_cpu_baseline)
        if rec is not None:
            for k in ("metric", "n_gpus", "higher_is_better", "vs_baseline", "data"):
                rec.pop(k, None)
            line["batch"] = rec
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------
BATCH_WORKLOAD = ("batched uneven mix: {count} systems, n log-uniform in [1k, {nmax}], even ones 2D-Laplacian "
                  "Cholesky factors (grid side round(sqrt n), full band), odd ones random diagonally dominant (the "
                  "irregular generator, Poisson mean U[4,16]), RHS U{{1..16}} per system, b = U x*, seed 2")


def batch_fp64_bytes(M):
    """Algorithmic bytes of one FP64 pass over the whole mix (the per-system FP64 unit summed)."""
    return int(np.sum(12 * M.nnz + 4 * (M.n.astype(np.int64) + 1) + 16 * M.n.astype(np.int64) * M.rhs))


def batch_cpu_sample(M, budget_s=12.0, seed=0):
    """Serial backward substitution (the reference's base_gauss_upper, else the oracle's
    restatement) over a seeded random sample of the systems until budget_s; returns the
    projected solves/s for the whole mix (count / (mean time per system * count))."""
    from oracle import oracle
    oracle.build()
    R = oracle.ref()
    order = np.random.default_rng(seed).permutation(M.count)
    t_sum, done, work_done = 0.0, 0, 0.0
    work = M.nnz.astype(np.float64) * M.rhs
    t0 = time.perf_counter()
    for s in order:
        m, _, b = M.system(int(s))
        r = int(M.rhs[s])
        bcm = np.ascontiguousarray(np.asarray(b).reshape(m.n, r).T).reshape(-1)
        x = np.zeros(m.n * r)
        rpu = m.row_ptr.astype(np.uint64)
        col = np.ascontiguousarray(m.col)
        val = np.ascontiguousarray(m.val)
        t1 = time.perf_counter()
        if R is not None:
            R.ref_base_gauss_upper(m.n, val, rpu, col, x, bcm, r)
        else:
            oracle.lib().orc_base_gauss_upper(m.n, val, rpu, col, x, bcm, r)
        t_sum += time.perf_counter() - t1
        work_done += work[s]
        done += 1
        if time.perf_counter() - t0 > budget_s and done >= 8:
            break
    # project by work (nnz x rhs): the sample's time per unit of work times the mix's work
    est_total = t_sum / work_done * float(np.sum(work))
    return {"value": M.count / est_total, "unit": "solves/s", "cores": 1,
            "kind": "reference" if R is not None else "port",
            "sample": f"serial base_gauss_upper on {done} randomly chosen systems of the mix ({t_sum:.1f} s), "
                      f"projected to all {M.count} by nnz x rhs ({os.uname().machine} host)"}


_FP64 = {}


def fp64_pipe(device=0):
    """The FP64 pipe of this GPU, measured by the library (sptrsv_measure_fp64): G FMA/s of
    independent FMA chains over every SM (the ceiling of the FP64-pipe-bound kernels: the residual,
    the exact FP64 panels) and SM cycles per dependent FMA (the floor of one dependency hop of an
    exact FP64 solve)."""
    if device not in _FP64:
        import sptrsv_gb300 as sp
        g, c = sp.measure_fp64(device)
        _FP64[device] = {"gfma_per_s": g, "dep_fma_cycles": c, "source": "sptrsv_measure_fp64 in this run"}
    return _FP64[device]


def fp64_rate(fma, prof_kind, device=0):
    """FMAs per launch and the rate of the kind's first launch (every system active), also as a
    fraction of the measured FP64 rate."""
    if not prof_kind:
        return {"fma_per_launch": fma, "gfma_per_s": None}
    g = fma / (prof_kind[2] * 1e-3) / 1e9
    ref = fp64_pipe(device)["gfma_per_s"]
    return {"fma_per_launch": fma, "gfma_per_s": g, "frac_of_measured_fp64": g / ref,
            "measured_fp64_gfma_per_s": ref}


def batch_errors_vs_serial(M, mine, B, xs_mode, sched, count=16, seed=7):
    """Errors of both modes against the reference's serial FP64 solve (the oracle's restatement of
    core.cpp:18-32) on a seeded sample of `count` of this rank's systems that always holds the
    largest banded and the largest random system: relative residual ||B - U X||_F / ||B||_F, max
    elementwise relative error (components below 1e-12 measured against 1e-12) and the
    term-relative error (against max(|x_i|, (|b_i| + sum_j |U_ij x_j|) / |U_ii|), the size of what
    component i is summed from).  Maxima over the sample per mode and per schedule kind."""
    from oracle import oracle
    idx = np.asarray(mine)
    kind = M.kind[idx]
    big = [int(idx[np.flatnonzero(kind == k)[np.argmax(M.n[idx][kind == k])]]) for k in (0, 1) if np.any(kind == k)]
    rest = [int(v) for v in np.random.default_rng(seed).permutation(idx) if int(v) not in big]
    pick = big + rest[:max(0, count - len(big))]
    where = {int(g): k for k, g in enumerate(idx)}
    parts = {mode: B.split(x) for mode, x in xs_mode.items()}
    worst = {}
    per = []
    for g in pick:
        m, _, b = M.system(g)
        r = int(M.rhs[g])
        rpu = m.row_ptr.astype(np.uint64)
        col, val = np.ascontiguousarray(m.col), np.ascontiguousarray(m.val)
        bcm = np.ascontiguousarray(np.asarray(b).reshape(m.n, r).T).reshape(-1)
        ref = oracle.base_gauss_upper(rpu, col, val, bcm, r)
        rec = {"system": g, "n": int(m.n), "rhs": r, "kind": "banded" if M.kind[g] == 0 else "random",
               "schedule": int(sched[where[g]])}
        for mode, pl in parts.items():
            xcm = np.ascontiguousarray(np.asarray(pl[where[g]]).T).reshape(-1)
            e = {"rel_residual": oracle.rel_residual(rpu, col, val, xcm, bcm, r),
                 "max_elem_rel_error": oracle.max_elem_rel_error(ref, xcm, 1e-12),
                 "term_rel_error": oracle.term_rel_error(rpu, col, val, ref, xcm, bcm, r)}
            rec[mode] = e
            names = {v: k for k, v in __import__("sptrsv_gb300").BATCH_SCHED.items()}
            key = mode if mode == "plain" else "chosen_" + names.get(int(sched[where[g]]), str(int(sched[where[g]])))
            w = worst.setdefault(key, {k: 0.0 for k in e})
            for k, v in e.items():
                w[k] = max(w[k], v)
        per.append(rec)
    return {"oracle": "serial base_gauss_upper (core.cpp:18-32), FP64", "sampled": len(pick),
            "includes": "the largest banded and the largest random system", "max_by_form": worst, "systems": per}


def batch_record(args, dist, steps, warmup, with_cpu=True, sample_errors=True):
    """Measures the batched mix (the 512-system uneven workload) and returns its JSON record on rank 0
    (None elsewhere)."""
    import ctypes
    import sptrsv_gb300 as sp
    from sptrsv_gb300 import gen
    from sptrsv_gb300 import selector as sel
    L = sp._lib.lib()
    t_gen = time.time()
    M = gen.mix(count=args.count, seed=2, nmin=1000, nmax=args.nmax)
    t_gen = time.time() - t_gen
    # several GPUs: each rank solves its own LPT share of the systems (by nnz x rhs); no collective
    from sptrsv_gb300.shard import lpt_partition, subset_arena, system_costs
    mine = lpt_partition(system_costs(M.nnz, M.rhs), dist.ws)[dist.rank] if dist.ws > 1 else list(range(M.count))
    l_n, l_rhs, l_rp, l_col, l_val, l_b, l_xs = (subset_arena(M, mine) if dist.ws > 1 else
                                                 (M.n, M.rhs, M.row_ptr, M.col, M.val, M.b, M.xstar))
    l_nnz = M.nnz[mine]
    B = sp.Batch(l_n, l_rhs, l_rp, l_col, l_val, device=dist.local)
    info = B.info()
    count_l = len(mine)
    # chosen schedules: the trained selector's picks when its weights are present, else the analysis default
    wpath = os.path.join(ROOT, "sptrsv_gb300", "data", "selector_gb300.npz")
    picked_by = "analysis default"
    if os.path.exists(wpath):
        mlp = sel.Mlp.load(wpath, device=dist.local)
        B.schedule = sel.batch_schedule(B, mlp)
        picked_by = "MLP selector"
    sched = B.schedule
    s = sp.Solver(dist.local)
    h = s.handle
    nb = 8 * int(info["x_elems"])
    d_b, d_x = ctypes.c_void_p(), ctypes.c_void_p()
    assert L.sptrsv_device_alloc(h, nb, ctypes.byref(d_b)) == 0
    assert L.sptrsv_device_alloc(h, nb, ctypes.byref(d_x)) == 0
    L.sptrsv_copy_h2d(h, d_b, l_b.ctypes.data, nb)
    assert s.sync() == 0

    def run(mode, steps):
        ms, ks = [], []
        for _ in range(steps):
            B.timer_begin()
            B.solve_device(d_b.value, d_x.value, mode)
            ms.append(B.timer_end())
            ks.append(B.sync())
        return ms, ks

    # correctness of both modes before timing
    xs_mode = {}
    worst = {}
    for mode in ("plain", "chosen"):
        run(mode, 1)
        x = np.empty(int(info["x_elems"]))
        L.sptrsv_copy_d2h(h, x.ctypes.data, d_x, nb)
        assert s.sync() == 0
        worst[mode] = float(np.max(np.abs(x - l_xs)))
        xs_mode[mode] = x
    st = B.stats()
    if np.any(st["status"] != 0) or not np.all(st["rel"][(sched != 0) & (sched != 4)] <= RES_TOL):
        raise SystemExit("batched chosen form missed the tolerance")
    run("chosen", warmup)
    clocks = Clocks(dist.local)
    clocks.start()
    dist.barrier()
    ms, ks = run("chosen", steps)
    ck = clocks.stop()
    dist.barrier()
    total_s = dist.max(sum(ms) / 1e3)
    value = args.count * steps / total_s  # every system of the mix, over the slowest rank
    run("plain", 1)
    psteps = max(2, min(steps, 3))
    pms, _ = run("plain", psteps)
    plain_sps = args.count * psteps / dist.max(sum(pms) / 1e3)
    # e2e: host b -> device, solve, x -> host, per step (pinned host buffers)
    hb, hx = ctypes.c_void_p(), ctypes.c_void_p()
    assert L.sptrsv_host_alloc(h, nb, ctypes.byref(hb)) == 0
    assert L.sptrsv_host_alloc(h, nb, ctypes.byref(hx)) == 0
    ctypes.memmove(hb, l_b.ctypes.data, nb)
    e2e_ms = []
    for k in range(warmup + steps):
        B.timer_begin()
        B.solve_host(hb.value, hx.value, "chosen")
        t = B.timer_end()
        B.sync()
        if k >= warmup:
            e2e_ms.append(t)
    e2e_value = args.count * steps / dist.max(sum(e2e_ms) / 1e3)
    # per-kernel device times: the same solve replayed from the host with events around every kernel
    prof = B.profile(d_b.value, d_x.value, "chosen")
    pplain = B.profile(d_b.value, d_x.value, "plain")
    mixed = (sched != 0) & (sched != 4)
    nn = l_n.astype(np.int64)
    lr = l_rhs.astype(np.int64)
    res_bytes = int(np.sum((12 * l_nnz + 4 * (nn + 1) + 20 * nn * lr)[mixed]))   # CSR + b, x read, r32 written
    res_fma = int(np.sum((l_nnz * lr)[mixed]))
    jac = sched == 1
    jac_bytes = int(np.sum((8 * (l_nnz - nn) + 4 * (nn + 1) + 16 * nn * lr)[jac]))
    info = B.info()  # with the schedules' work lists built
    p64 = sched == 4
    p64_bytes = int(8 * info["g_entries_f64"] + np.sum((4 * (nn + 1) + 16 * nn * lr)[p64]))  # G once, b, x
    dom = max(prof, key=lambda k: prof[k][0])
    dom_bytes = {"residual_f64": res_bytes, "jacobi_sweep": jac_bytes, "panels_f64": p64_bytes}.get(dom)
    dom_first = prof[dom][2]
    cpu = None
    if dist.rank == 0 and with_cpu:
        try:
            cpu = batch_cpu_sample(M)
        except Exception as e:
            cpu = {"value": None, "unit": "solves/s", "error": str(e)[:200]}
    errs = None
    if dist.rank == 0 and sample_errors:
        try:
            errs = batch_errors_vs_serial(M, mine, B, xs_mode, sched)
        except Exception as e:  # reported, never required
            errs = {"error": str(e)[:200]}
    del xs_mode
    L.sptrsv_host_free(h, hb)
    L.sptrsv_host_free(h, hx)
    L.sptrsv_device_free(h, d_b)
    L.sptrsv_device_free(h, d_x)
    B.close()
    s.close()
    if dist.rank != 0:
        M.close()
        return None
    fb = batch_fp64_bytes(M)
    peak, peak_src = measured_peak()
    ms_step = 1e3 * total_s / steps
    counts = {k: int(np.sum(sched == v)) for k, v in sp.BATCH_SCHED.items()}
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": dist.ws, "steps": steps,
        "warmup": warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": BATCH_WORKLOAD.format(count=args.count, nmax=args.nmax), "systems": args.count,
                   "rows": int(np.sum(M.n)), "nnz": int(np.sum(M.nnz)), "rhs_columns": int(np.sum(M.rhs)),
                   "rank0_systems": count_l, "schedules": counts, "picked_by": picked_by, "generation_s": t_gen,
                   "panel_products": {"tc": "tensor cores (BF16 digit slices, FP64-accurate)",
                                      "df": "double-FP32 on the FP32 pipes (FP64-accurate)"}.get(args.panels, "FP64 FMAs"),
                   "l2": "no flush: the arena (%.1f GB) is far larger than L2" % (fb / 1e9),
                   "parallelism": f"systems sharded over {dist.ws} GPU(s) by LPT on nnz x rhs"},
        "solve_unit": "one system with all its right-hand sides",
        "hbm_gbs": fb / (ms_step * 1e-3) / 1e9,
        "us_per_solve": 1e3 * ms_step / args.count,
        "gflops": float(np.sum((2 * (M.nnz - M.n) + M.n) * M.rhs)) / (ms_step * 1e-3) / 1e9,
        "plain_fp64_syncfree": {"solves_per_s": plain_sps, "ms_per_batch": 1e3 * args.count / plain_sps,
                                "hbm_gbs": fb * plain_sps / args.count / 1e9},
        "speedup_vs_plain": value / plain_sps,
        "max_abs_err_vs_xstar": worst,
        "refine_steps_max": int(np.max(st["steps"])), "rel_residual_max": float(np.max(st["rel"])),
        "refine_steps_by_schedule": {k: np.bincount(st["steps"][sched == v], minlength=4).tolist()
                                     for k, v in sp.BATCH_SCHED.items() if np.any(sched == v)},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb},
        "roofline": ({"bound": "hbm", "kernel": {"residual_f64": "k_b_residual", "jacobi_sweep": "k_b_jacobi",
                                                 "panels_f64": "k_panels64"}[dom],
                      "achieved": dom_bytes / (dom_first * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                      "frac": dom_bytes / (dom_first * 1e-3) / 1e9 / peak, "peak_source": peak_src, "traffic": None,
                      "algorithmic_bytes_per_launch": dom_bytes, "launch_ms": dom_first,
                      "note": "first launch (every system of the kernel's schedule active)"}
                     if dom_bytes else
                     {"bound": "hbm", "kernel": dom, "achieved": fb / (ms_step * 1e-3) / 1e9, "peak": peak,
                      "unit": "GB/s", "frac": fb / (ms_step * 1e-3) / 1e9 / peak, "peak_source": peak_src,
                      "traffic": None, "algorithmic_bytes_per_launch": fb, "note": "whole solve"}),
        "fp64_residual": fp64_rate(res_fma, prof.get("residual_f64"), dist.local),
        "fp64_panels": dict(fp64_rate(info["g_fma_f64"], prof.get("panels_f64"), dist.local),
                            g_entries=info["g_entries_f64"]),
        "kernel_profile_chosen": {k: {"ms": v[0], "launches": v[1]} for k, v in prof.items()},
        "kernel_profile_plain": {k: {"ms": v[0], "launches": v[1]} for k, v in pplain.items()},
        "gpu_launches": int(sum(ks)),
        "clocks": ck,
        "cpu_baseline": cpu,
        "vs_oracle": errs,
    }
    M.close()
    return line


def run_batch(args, dist):
    line = batch_record(args, dist, args.steps, args.warmup, not args.no_cpu_baseline)
    if line is not None:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------
def run_supernodal(args, dist):
    """The 3D-Laplacian nested-dissection factor (40^3, supernodes 8-400): device time per solve
    (CUDA events, L2 flushed, best of `steps`) of the FP64 supernodal schedule, the mixed one
    (BF16x3 tensor-core panels + FP64 refinement) and the plain FP64 sync-free schedule, at
    1, 8, 32 and 128 right-hand sides, beside the serial CPU solve."""
    import ctypes
    import sptrsv_gb300 as sp
    from sptrsv_gb300 import gen
    from oracle import oracle
    if dist.rank != 0:
        return
    L = sp._lib.lib()
    # the factor from the library's GPU multifrontal Cholesky (the host generator's factor matches
    # it to 1e-12, tests/test_gpu_supernodal_full.py); the second run is the one reported
    t_gen = time.time()
    m = gen.laplace3d_nd_cholesky_gpu(40, device=dist.local)
    t_gen = time.time() - t_gen
    t_fac = time.time()
    m = gen.laplace3d_nd_cholesky_gpu(40, device=dist.local)
    t_fac = time.time() - t_fac
    s = sp.Solver(dist.local)
    s.analyse(m.row_ptr, m.col, m.val).set_supernodes(m.snodes)
    h = s.handle
    rows = []
    pad = None  # the padded format of the BLAS-supernodal CPU path (core.cpp:136-161), built once
    rpu = m.row_ptr.astype(np.uint64)
    for rhs in [int(v) for v in args.rhs.split(",")]:
        b = gen.uniform(3 + rhs, m.n * rhs)
        ref = oracle.base_gauss_upper(rpu, m.col, m.val, b, rhs)
        # two correct FP64 solves differing only in summation order lie this far apart elementwise
        floor = oracle.max_elem_rel_error(ref, oracle.base_gauss_upper_rev(rpu, m.col, m.val, b, rhs), 1e-12)
        nb = 8 * m.n * rhs
        d_b, d_x = ctypes.c_void_p(), ctypes.c_void_p()
        assert L.sptrsv_device_alloc(h, nb, ctypes.byref(d_b)) == 0
        assert L.sptrsv_device_alloc(h, nb, ctypes.byref(d_x)) == 0
        L.sptrsv_copy_h2d(h, d_b, b.ctypes.data, nb)
        row = {"rhs": rhs, "reorder_floor_elem_err": floor}
        for name, o, reps in (("fp64_supernodal", sp.make_opts(schedule="supernodal"), args.steps),
                              ("mixed_supernodal_bf16x3", sp.make_opts(schedule="supernodal", precision="mixed"),
                               args.steps),
                              # the plain FP64 sync-free kernels once per column (this factor's rows
                              # are long: faster than the RHS-tiled warp kernel)
                              ("plain_fp64_syncfree", sp.make_opts(schedule="syncfree_block"), 1 if rhs > 1 else 3),
                              ("plain_fp64_window", sp.make_opts(schedule="syncfree_window"), 1 if rhs > 1 else 3)):
            x = np.empty(m.n * rhs)
            best = None
            for k in range(1 + reps):
                L.sptrsv_flush_l2(h)
                L.sptrsv_timer_begin(h)
                rc = L.sptrsv_solve(h, ctypes.byref(o), d_b, d_x, rhs, sp.COL_MAJOR)
                fms = ctypes.c_float()
                L.sptrsv_timer_end(h, ctypes.byref(fms))
                if rc or s.sync():
                    raise SystemExit(f"{name} failed")
                if k > 0:
                    best = fms.value if best is None else min(best, fms.value)
            L.sptrsv_copy_d2h(h, x.ctypes.data, d_x, nb)
            s.sync()
            row[name] = {"ms": best, "elem_err": oracle.max_elem_rel_error(ref, x, 1e-12),
                         "term_rel_err": oracle.term_rel_error(rpu, m.col, m.val, ref, x, b, rhs),
                         "rel_residual": oracle.rel_residual(rpu, m.col, m.val, x, b, rhs)}
        t0 = time.perf_counter()
        oracle.base_gauss_upper(rpu, m.col, m.val, b, rhs)
        row["cpu_serial_ms"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        oracle.supernodal_upper(m.snodes, rpu, m.col, m.val, b, rhs)
        row["cpu_supernodal_ms"] = 1e3 * (time.perf_counter() - t0)
        if pad is None:
            pad = oracle.ccs2ccs_pad(m.snodes, rpu, m.col, m.val)
        t0 = time.perf_counter()
        oracle.supernodal_blas_upper(m.snodes, pad[0], pad[1], pad[2], b, rhs)
        row["cpu_supernodal_blas_ms"] = 1e3 * (time.perf_counter() - t0)
        # the same algorithm with its dgemm / dtrsm on numpy's OpenBLAS, every host core
        oracle.supernodal_blas_upper_openblas(m.snodes, pad[0], pad[1], pad[2], b, 1)
        t0 = time.perf_counter()
        if oracle.supernodal_blas_upper_openblas(m.snodes, pad[0], pad[1], pad[2], b, rhs) is not None:
            row["cpu_supernodal_openblas_ms"] = 1e3 * (time.perf_counter() - t0)
        rows.append(row)
        L.sptrsv_device_free(h, d_b)
        L.sptrsv_device_free(h, d_x)
    info = s.info()
    print(json.dumps({"workload": "supernodal: 7-point 3D Laplacian Cholesky factor, 40^3 grid, nested dissection "
                                  "(8^3 leaves), supernodes <= 400 rows",
                      "cpu": f"{cpu_model()}: serial, supernodal and BLAS-supernodal restatements of core.cpp on 1 "
                             "thread (the last with plain-loop dgemm/dtrsm); 'MKL-supernodal -> OpenBLAS-supernodal': "
                             "supernodal_blas_upper with its dgemm/dtrsm on numpy's OpenBLAS "
                             f"({(oracle.cblas64() or ['absent'])[0]}) with its default thread count, "
                             f"{os.environ.get('OPENBLAS_NUM_THREADS', os.cpu_count())} threads (MKL is not on the host)",
                      "elementwise": "elem_err: max |x - ref| / max(|ref|, 1e-12); term_rel_err: against "
                                     "max(|ref_i|, (|b_i| + sum_j |U_ij ref_j|) / |U_ii|); reorder_floor_elem_err: "
                                     "elem_err of the serial solve summed in reverse order",
                      "n": m.n, "nnz": m.nnz, "supernodes": int(len(m.snodes) - 1), "max_level": info["max_level"],
                      "panels": args.panels, "generation_s": t_gen,
                      "factor": {"how": "sptrsv_factor_multifrontal: host symbolic step, fronts assembled and "
                                        "factored on the GPU in FP64", "seconds": t_fac},
                      "rows": rows}), flush=True)


def run_dropin(args, dist):
    """The reference-signature entry point base_gauss_upper (core.h:10) on three systems: the
    64 x 64 grid Laplacian factor (n = 4,096, the reference's own CPU-runnable case), the
    256 x 256 one and the 2M-row irregular system.  Per system: the solve time the call returns
    (device events around the solve, as the reference reports its kernel time), the wall time of
    the whole call (upload, analysis, solve, copies), the serial CPU solve, and the elementwise
    error against it."""
    if dist.rank != 0:
        return
    import sptrsv_gb300 as sp
    from sptrsv_gb300 import gen
    from oracle import oracle
    cases = [("band 64x64 grid factor (n=4,096)", lambda: gen.band_laplace_case()),
             ("band 256x256 grid factor (n=65,536)", lambda: (lambda mm: (mm,) + gen.system(mm, 0))(
                 gen.laplace2d_cholesky(256))),
             ("irregular 2M", lambda: gen.irregular_case(args.n))]
    rows = []
    for name, make in cases:
        m, xs, b = make()
        rpu = m.row_ptr.astype(np.uint64)
        cpu_s = None
        for _ in range(3):  # best of three, warm
            t0 = time.perf_counter()
            ref = oracle.base_gauss_upper(rpu, m.col, m.val, b, 1)
            el = time.perf_counter() - t0
            cpu_s = el if cpu_s is None else min(cpu_s, el)
        best, wall = None, None
        x = np.zeros(m.n)
        for k in range(max(2, min(args.steps, 5)) + 1):
            x = np.zeros(m.n)
            t0 = time.perf_counter()
            secs = sp.base_gauss_upper(m.n, m.val, rpu, m.col, x, b, 1)
            w = time.perf_counter() - t0
            if secs < 0:
                raise SystemExit(f"base_gauss_upper failed on {name}: {secs}")
            if k > 0:
                best = secs if best is None else min(best, secs)
                wall = w if wall is None else min(wall, w)
        rows.append({"system": name, "n": m.n, "nnz": m.nnz, "solve_ms": 1e3 * best, "call_wall_ms": 1e3 * wall,
                     "cpu_serial_ms": 1e3 * cpu_s, "solve_speedup_vs_cpu": cpu_s / best,
                     "max_elem_rel_error": oracle.max_elem_rel_error(ref, x, 1e-12),
                     "rel_residual": oracle.rel_residual(rpu, m.col, m.val, x, b, 1)})
    print(json.dumps({"workload": "drop-in base_gauss_upper (core.h:10) against the serial CPU solve",
                      "cpu": f"{cpu_model()}, 1 thread (oracle restatement of base_gauss_upper)",
                      "rows": rows}), flush=True)


def run_factor(args, dist):
    """The multifrontal Cholesky A = U^T U of the 7-point 3D Laplacian on a grid^3 grid under
    nested dissection (8^3 leaves, supernodes <= 400 rows) through sptrsv_factor_multifrontal:
    wall time of the call (host symbolic step + GPU numeric step, U left on the device; best of
    `steps` after `warmup` calls), the two steps apart, the copy of U to host memory timed apart
    (sptrsv_factor_copy), and the factor's FLOPs (sum over columns of L of c_j^2, c_j the
    column's entries) over the numeric step against the measured FP64 pipe.  Beside it the host
    generator's factor of the same matrix and fronts (numpy/scipy dense fronts, LAPACK on the
    host's OpenBLAS) timed once, and the largest difference between the two factors."""
    import ctypes
    import sptrsv_gb300 as sp
    from sptrsv_gb300 import gen
    if dist.rank != 0:
        return
    L = sp._lib.lib()
    g = args.grid
    rp, col, val, fs, fp, _ = gen.laplace3d_nd_matrix(g)
    n = len(rp) - 1
    times = []
    for k in range(max(3, args.warmup) + args.steps):
        h = ctypes.c_void_p()
        t0 = time.perf_counter()
        rc = L.sptrsv_factor_multifrontal(dist.local, n, rp, col, val, len(fs) - 1, fs, fp, 400, ctypes.byref(h))
        wall = time.perf_counter() - t0
        if rc:
            raise SystemExit("sptrsv_factor_multifrontal: " + sp.status_string(rc))
        sym, num = ctypes.c_double(), ctypes.c_double()
        L.sptrsv_factor_times(h, ctypes.byref(sym), ctypes.byref(num))
        nn, nnz, nsn = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int()
        L.sptrsv_factor_info(h, ctypes.byref(nn), ctypes.byref(nnz), ctypes.byref(nsn))
        urp = np.empty(n + 1, dtype=np.int64)
        ucol = np.empty(nnz.value, dtype=np.int32)
        uval = np.empty(nnz.value, dtype=np.float64)
        t0 = time.perf_counter()
        L.sptrsv_factor_copy(h, urp, ucol, uval, np.empty(nsn.value + 1, dtype=np.int32))
        copy = time.perf_counter() - t0
        if k >= max(3, args.warmup):
            times.append((wall, sym.value, num.value, copy))
        L.sptrsv_factor_free(h)
    wall, sym, num, copy = min(times)
    c = np.diff(urp).astype(np.float64)
    flops = float((c * c).sum())
    pipe = fp64_pipe(dist.local)
    rec = {"workload": f"factor: 7-point 3D Laplacian, {g}^3 grid, nested dissection (8^3 leaves), fronts "
                       f"{len(fs) - 1}, supernodes <= 400 rows",
           "metric": "factor wall seconds (host symbolic + GPU numeric, U on the device)", "unit": "s",
           "higher_is_better": False,
           "n": n, "nnz_A": int(rp[-1]), "nnz_U": int(nnz.value), "supernodes": int(nsn.value),
           "steps": len(times), "value": wall, "symbolic_s": sym, "numeric_s": num, "copy_to_host_s": copy,
           "all_wall_s": [t[0] for t in times],
           "update_form": ("FP64 FMAs" if os.environ.get("SPTRSV_FACTOR_UPDATE") == "fp64" else
                           "tensor cores (BF16 digit slices, FP64-accurate) for fronts with >= 256 rows below "
                           "the panel, FP64 FMAs for the rest"),
           "flops": flops, "numeric_gflop_per_s": flops / num / 1e9,
           "frac_of_measured_fp64": flops / num / 1e9 / (2.0 * pipe["gfma_per_s"]),
           "measured_fp64_gfma_per_s": pipe["gfma_per_s"],
           "rate_note": "FLOPs of the FP64 factorisation (sum of c_j^2) over the numeric step; with the "
                        "tensor-core updates this is an FP64-equivalent rate and can exceed the FP64 pipe"}
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        hm = gen.laplace3d_nd_cholesky(g)
        rec["cpu_baseline"] = {"value": time.perf_counter() - t0, "unit": "s", "kind": "port",
                               "cores": int(os.environ.get("OPENBLAS_NUM_THREADS", os.cpu_count())),
                               "sample": f"gen.laplace3d_nd_cholesky({g}): the same fronts as dense numpy/scipy "
                                         "blocks (LAPACK/BLAS on numpy's OpenBLAS), one run"}
        rec["max_abs_diff_vs_host"] = float(np.max(np.abs(hm.val - uval)))
        rec["max_abs_U"] = float(np.max(np.abs(uval)))
    print(json.dumps(rec), flush=True)


def apply_options(args):
    """Process-wide choices the command line makes before anything is built."""
    global PLAIN_SCHEDULE
    if args.impl == "ours":
        import sptrsv_gb300 as sp
        sp.set_panels_mode(args.panels)
        if args.plain_schedule:
            PLAIN_SCHEDULE = args.plain_schedule


def main():
    args = parse()
    dist = Dist()
    try:
        apply_options(args)
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.workload == "batch":
            run_batch(args, dist)
        elif args.workload == "supernodal":
            run_supernodal(args, dist)
        elif args.workload == "dropin":
            run_dropin(args, dist)
        elif args.workload == "factor":
            run_factor(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()

"""The learned schedule selector: an MLP that predicts every candidate schedule's log runtime from
a matrix's features and picks the fastest, with the exhaustive autotuner as its fallback and its
judge.

* ``Mlp``: the network (include/sptrsv_gb300.h, sptrsv_mlp_*), trained and evaluated on the GPU by
  the library's own forward / backward / Adam kernels;
* ``build_dataset``: times every candidate of the autotuner's table (sptrsv_autotune) on seeded
  matrices from the three generators (banded Laplacian factors cut into 64-row skyline panels,
  random irregular factors, random supernodal factors) with a random RHS count, next to their
  features (sptrsv_features);
* ``train`` / ``evaluate``: fit on one part, report on held-out matrices the regret against the
  exhaustive tuner's best (t_pick / t_best - 1) and the speed-up over a fixed default schedule
  (the single candidate with the best geometric-mean time on the training part);
* ``batch_schedule``: the batched path's per-system schedules from the network's picks.

The network only chooses a schedule; every solve's arithmetic is the chosen schedule's own.

Command line (one GPU): ``python -m sptrsv_gb300.selector build --count 2200 --out FILE`` builds
a timing dataset; ``python -m sptrsv_gb300.selector eval --data FILE`` trains and reports.
"""
import ctypes
import math
import os
import time

import numpy as np

from . import _lib, N_CANDIDATES, N_FEATURES, Solver, SptrsvError, candidate, _check
from . import gen

DIMS = (N_FEATURES, 64, 64, N_CANDIDATES)
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "tuning_gb300.npz")
KINDS = ("band", "random", "supernodal")


class Mlp:
    """FP32 MLP in -> h1 -> h2 -> out on the GPU (sptrsv_mlp_*)."""

    def __init__(self, dims=DIMS, seed=0, device=0):
        self.dims = tuple(int(d) for d in dims)
        h = ctypes.c_void_p()
        _check(_lib.lib().sptrsv_mlp_create(ctypes.byref(h), int(device), *self.dims, int(seed)), "mlp_create")
        self._h = h
        self.mean = np.zeros(self.dims[0], dtype=np.float32)
        self.scale = np.ones(self.dims[0], dtype=np.float32)

    def close(self):
        if self._h:
            _lib.lib().sptrsv_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self):
        return int(_lib.lib().sptrsv_mlp_num_params(self._h))

    @property
    def params(self):
        p = np.zeros(self.num_params, dtype=np.float32)
        _check(_lib.lib().sptrsv_mlp_get_params(self._h, p), "mlp_get_params")
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params
        _check(_lib.lib().sptrsv_mlp_set_params(self._h, p), "mlp_set_params")

    def set_norm(self, mean, scale):
        self.mean = np.ascontiguousarray(mean, dtype=np.float32)
        self.scale = np.ascontiguousarray(scale, dtype=np.float32)
        _check(_lib.lib().sptrsv_mlp_set_norm(self._h, self.mean, self.scale), "mlp_set_norm")

    def fit_norm(self, X):
        X = np.asarray(X, dtype=np.float64)
        sd = X.std(0)
        self.set_norm(X.mean(0), np.where(sd > 1e-6, 1.0 / np.maximum(sd, 1e-6), 1.0))

    def grad(self, X, Y, M):
        X, Y, M = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, Y, M))
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _check(_lib.lib().sptrsv_mlp_grad(self._h, X.shape[0], X, Y, M, g, loss), "mlp_grad")
        return float(loss[0]), g

    def train(self, X, Y, M, epochs=300, batch=128, lr=2e-3, seed=0):
        X, Y, M = (np.ascontiguousarray(a, dtype=np.float32) for a in (X, Y, M))
        losses = np.zeros(int(epochs), dtype=np.float32)
        _check(_lib.lib().sptrsv_mlp_train(self._h, X.shape[0], X, Y, M, int(epochs), int(batch), float(lr),
                                           int(seed), losses), "mlp_train")
        return losses

    def predict(self, X):
        X = np.ascontiguousarray(np.atleast_2d(X), dtype=np.float32)
        out = np.zeros((X.shape[0], self.dims[3]), dtype=np.float32)
        _check(_lib.lib().sptrsv_mlp_predict(self._h, X.shape[0], X, out), "mlp_predict")
        return out

    def launches(self):
        return int(_lib.lib().sptrsv_mlp_launches(self._h))

    def save(self, path):
        np.savez(path, params=self.params, mean=self.mean, scale=self.scale, dims=np.array(self.dims))

    @classmethod
    def load(cls, path, device=0):
        d = np.load(path)
        m = cls(tuple(d["dims"]), device=device)
        m.params = d["params"]
        m.set_norm(d["mean"], d["scale"])
        return m


# ---------------------------------------------------------------------------------------------
# dataset

def sample_specs(count, seed, nmax=2_000_000):
    """Seeded matrix specs (numpy PCG64): kind round-robin over KINDS; band: grid side U{16..64};
    random: n log-uniform [1k, nmax], Poisson mean U[2, 32], band log-uniform [8, 512];
    supernodal: n log-uniform [1k, nmax/4], widths U{1..w} with w log-uniform [4, 128]; RHS 1 with
    probability 1/2, else U{2..16}."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(count):
        kind = KINDS[k % 3]
        rhs = 1 if rng.random() < 0.5 else int(rng.integers(2, 17))
        ms = int(rng.integers(1, 2 ** 62))
        if kind == "band":
            specs.append(dict(kind=0, g=int(rng.integers(16, 65)), n=0, mean=0.0, band=0, wmax=0, rhs=rhs, seed=ms))
        elif kind == "random":
            n = int(round(math.exp(rng.uniform(math.log(1000), math.log(nmax)))))
            band = int(round(math.exp(rng.uniform(math.log(8), math.log(512)))))
            specs.append(dict(kind=1, g=0, n=n, mean=float(rng.uniform(2, 32)), band=band, wmax=0, rhs=rhs, seed=ms))
        else:
            n = int(round(math.exp(rng.uniform(math.log(1000), math.log(max(2000, nmax // 4))))))
            wmax = int(round(math.exp(rng.uniform(math.log(4), math.log(128)))))
            specs.append(dict(kind=2, g=0, n=n, mean=float(rng.uniform(2, 16)), band=64, wmax=wmax, rhs=rhs,
                              seed=ms))
    return specs


def make_matrix(spec):
    """(Csr, supernode partition or None) of a spec."""
    if spec["kind"] == 0:
        m = gen.laplace2d_cholesky(spec["g"])
        sn = np.unique(np.append(np.arange(0, m.n, 64), m.n)).astype(np.int32)
        return m, sn
    if spec["kind"] == 1:
        return gen.random_upper(spec["n"], spec["mean"], 0.9, spec["band"], spec["seed"]), None
    m = gen.supernodal_random(spec["n"], 1, spec["wmax"], spec["mean"], 0.8, spec["band"], spec["seed"])
    return m, m.snodes


def build_dataset(count, seed=7, nmax=2_000_000, cap_ms=20.0, reps=2, abort_ms=40.0, time_limit_s=None, out=None,
                  device=0, start=0, log=None):
    """Features and candidate timings (ms; inf where not applicable or failed) for specs
    [start, count) of sample_specs(count, seed, nmax).  A candidate still running after
    max(abort_ms, 20 x the best so far) is cancelled; its time is then a lower bound (C = 1)."""
    specs = sample_specs(count, seed, nmax)
    X, T, A, S, K, C = [], [], [], [], [], []
    t0 = time.time()
    with Solver(device) as s:
        for k in range(start, count):
            if time_limit_s is not None and time.time() - t0 > time_limit_s:
                break
            sp_ = specs[k]
            m, sn = make_matrix(sp_)
            s.analyse(m.row_ptr, m.col, m.val)
            if sn is not None:
                s.set_supernodes(sn)
            rhs = sp_["rhs"]
            f = s.features(rhs)
            try:
                _, ms, cens = s.autotune(rhs=rhs, cap_ms=cap_ms, reps=reps, abort_ms=abort_ms, with_censored=True)
            except SptrsvError:
                ms = np.full(N_CANDIDATES, np.inf, dtype=np.float32)
                cens = np.zeros(N_CANDIDATES, dtype=np.int32)
            app = np.array([s.applicable(c, rhs) for c in range(N_CANDIDATES)], dtype=np.int8)
            X.append(f)
            T.append(ms)
            A.append(app)
            S.append([sp_["kind"], sp_["g"], sp_["n"] or m.n, sp_["mean"], sp_["band"], sp_["wmax"], rhs, m.nnz])
            K.append(k)
            C.append(np.asarray(cens, dtype=np.int8))
            if log and (len(K) % 50 == 0):
                log("%d matrices, %.0f s" % (len(K), time.time() - t0))
            if out and len(K) % 100 == 0:
                _save(out, X, T, A, S, K, C, seed, nmax)
    if out:
        _save(out, X, T, A, S, K, C, seed, nmax)
    return dict(X=np.array(X, dtype=np.float32), T=np.array(T, dtype=np.float32), A=np.array(A, dtype=np.int8),
                S=np.array(S, dtype=np.float64), K=np.array(K, dtype=np.int32), C=np.array(C, dtype=np.int8))


def _save(path, X, T, A, S, K, C, seed, nmax):
    np.savez_compressed(path, X=np.array(X, dtype=np.float32), T=np.array(T, dtype=np.float32),
                        A=np.array(A, dtype=np.int8), S=np.array(S, dtype=np.float64), K=np.array(K, dtype=np.int32),
                        C=np.array(C, dtype=np.int8), seed=np.array([seed]), nmax=np.array([nmax]))


def merge(paths, out):
    """Concatenate dataset parts (disjoint spec ranges of one seed) into one file, in spec order."""
    parts = [load_dataset(p) for p in paths]
    keys = ("X", "T", "A", "S", "K", "C")
    d = {k: np.concatenate([p[k] for p in parts]) for k in keys}
    order = np.argsort(d["K"], kind="stable")
    d = {k: v[order] for k, v in d.items()}
    np.savez_compressed(out, **d, seed=parts[0]["seed"], nmax=parts[0]["nmax"])
    return d


def load_dataset(path=DATA):
    d = np.load(path)
    return {k: d[k] for k in d.files}


# ---------------------------------------------------------------------------------------------
# training and evaluation

def targets(T):
    """log(ms) targets and their mask (finite timings; a cancelled candidate's lower bound is kept
    as its target, which marks it as slow)."""
    M = np.isfinite(T).astype(np.float32)
    Y = np.where(M > 0, np.log(np.where(np.isfinite(T), np.maximum(T, 1e-6), 1.0)), 0.0).astype(np.float32)
    return Y, M


def fixed_default(T):
    """The single candidate with the best geometric-mean time among those that ran everywhere
    (else the one with the fewest failures)."""
    fin = np.isfinite(T)
    ok = np.all(fin, axis=0)
    logt = np.log(np.where(fin, np.maximum(T, 1e-6), 1.0))
    score = np.where(ok, logt.mean(0), np.inf)
    if np.all(~np.isfinite(score)):
        score = (~fin).sum(0) * 1e6 + np.where(fin, logt, 0).mean(0)
    return int(np.argmin(score))


def split(n, held_out, seed=0):
    perm = np.random.default_rng(seed).permutation(n)
    return np.sort(perm[held_out:]), np.sort(perm[:held_out])


def train(X, T, epochs=400, batch=128, lr=2e-3, seed=0, device=0):
    Y, M = targets(T)
    mlp = Mlp(seed=seed, device=device)
    mlp.fit_norm(X)
    losses = mlp.train(X, Y, M, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return mlp, losses


def pick(pred, applicable):
    """Index of the lowest predicted time among the applicable candidates, per row."""
    p = np.where(applicable > 0, pred, np.inf)
    return np.argmin(p, axis=1)


def evaluate(mlp, X, T, A, default_id):
    """Held-out report: the network's picks against the exhaustive tuner's best and the fixed
    default.  A pick that failed in tuning falls back to the tuner (its time = the tuner's best
    plus the pick's failed run is not counted) and is reported as a fallback."""
    pred = mlp.predict(X)
    pk = pick(pred, A)
    rows = np.arange(len(X))
    best = np.min(np.where(np.isfinite(T), T, np.inf), axis=1)
    valid = np.isfinite(best)
    tp = T[rows, pk]
    fallback = ~np.isfinite(tp)
    tp = np.where(fallback, best, tp)
    td = T[rows, default_id]
    td = np.where(np.isfinite(td), td, np.nan)
    v = valid & np.isfinite(td)
    regret = tp[valid] / best[valid] - 1.0
    return {
        "count": int(valid.sum()),
        "mean_regret": float(np.mean(regret)),
        "median_regret": float(np.median(regret)),
        "geomean_regret": float(np.exp(np.mean(np.log(tp[valid] / best[valid]))) - 1.0),
        "top1": float(np.mean(pk[valid] == np.argmin(np.where(np.isfinite(T), T, np.inf), axis=1)[valid])),
        "fallbacks": int(fallback[valid].sum()),
        "default_id": int(default_id),
        "default_geomean_regret": float(np.exp(np.mean(np.log(td[v] / best[v]))) - 1.0),
        "speedup_vs_default_geomean": float(np.exp(np.mean(np.log(td[v] / tp[v])))),
        "speedup_vs_default_total": float(np.sum(td[v]) / np.sum(tp[v])),
    }


# ---------------------------------------------------------------------------------------------
# the batched path's schedules from the network

# single-system candidate -> batched schedule (0 plain FP64, 1 Jacobi, 2 BF16x3 panels in the
# refinement, 3 FP32 sync-free, 4 exact FP64 panels): both supernodal candidates become the exact
# FP64 panels -- in the batch their products are split over CTAs and run beside the refinement,
# which measured faster than the BF16x3 panels' three refinement steps (190 ms against 281 ms for
# the 512-system mix with every banded system on one or the other); Jacobi stays Jacobi, the other
# mixed ones the FP32 pull, the other FP64 ones the plain FP64 pull
def batch_kind(cand_id):
    o = candidate(cand_id)
    if o.schedule == 6:
        return 4
    if o.precision == 0:
        return 0
    if o.schedule == 5:
        return 1
    return 3


def batch_schedule(batch, mlp):
    """Per-system batched schedules from the network's picks (restricted to what the batched path
    can run for that system)."""
    info = batch.info()
    sched = batch.schedule.copy()
    F = np.stack([batch.features(s) for s in range(batch.count)])
    pred = mlp.predict(F)
    order = np.argsort(pred, axis=1)
    for s in range(batch.count):
        rhs = int(batch.rhs[s])
        for c in order[s]:
            kind = batch_kind(int(c))
            o = candidate(int(c))
            if o.schedule in (2, 7) and rhs != 1:
                continue  # single-RHS candidates
            if kind == 1 and not info["ratio"][s] < 1.0:
                continue
            if kind in (2, 4) and F[s, 21] == 0.0:
                continue  # no panel structure
            if o.schedule == 6 and F[s, 21] == 0.0:
                continue
            sched[s] = kind
            break
    return sched


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(prog="python -m sptrsv_gb300.selector")
    sub = ap.add_subparsers(dest="cmd", required=True)
    b = sub.add_parser("build")
    b.add_argument("--count", type=int, default=2200)
    b.add_argument("--start", type=int, default=0)
    b.add_argument("--seed", type=int, default=7)
    b.add_argument("--nmax", type=int, default=2_000_000)
    b.add_argument("--cap-ms", type=float, default=20.0)
    b.add_argument("--reps", type=int, default=2)
    b.add_argument("--abort-ms", type=float, default=40.0)
    b.add_argument("--time-limit", type=float, default=None)
    b.add_argument("--out", required=True)
    mg = sub.add_parser("merge")
    mg.add_argument("parts", nargs="+")
    mg.add_argument("--out", required=True)
    e = sub.add_parser("eval")
    e.add_argument("--data", default=DATA)
    e.add_argument("--held-out", type=int, default=200)
    e.add_argument("--epochs", type=int, default=400)
    e.add_argument("--save", default=None, help="write the trained network (params, normalisation) here")
    a = ap.parse_args(argv)
    if a.cmd == "build":
        d = build_dataset(a.count, a.seed, a.nmax, a.cap_ms, a.reps, a.abort_ms, a.time_limit, a.out, start=a.start,
                          log=lambda s: print(s, flush=True))
        print(json.dumps({"matrices": int(len(d["K"])), "last_spec": int(d["K"][-1]) if len(d["K"]) else -1}))
    elif a.cmd == "merge":
        d = merge(a.parts, a.out)
        print(json.dumps({"matrices": int(len(d["K"]))}))
    else:
        d = load_dataset(a.data)
        tr, te = split(len(d["X"]), a.held_out)
        t0 = time.time()
        mlp, losses = train(d["X"][tr], d["T"][tr], epochs=a.epochs)
        t_train = time.time() - t0
        rep = evaluate(mlp, d["X"][te], d["T"][te], d["A"][te], fixed_default(d["T"][tr]))
        rep.update(train_matrices=int(len(tr)), held_out=int(len(te)), epochs=a.epochs, train_s=t_train,
                   first_loss=float(losses[0]), final_loss=float(losses[-1]), kernel_launches=mlp.launches())
        if a.save:
            mlp.save(a.save)
        print(json.dumps(rep))


if __name__ == "__main__":
    main()

"""Learned continued-fraction terminator.

A Lanczos run gives coefficients a_n, b_n; the spectral function is the
continued fraction over them, closed by the square-root terminator that
assumes the last coefficients repeat forever.  Here a 3-layer perceptron
(width 256, tanh) learns, from long runs that this engine produces on
synthetic ensembles, how the sequence continues: from a window of the last
48 normalised coefficients (a/sigma, b/sigma, sigma = (2 w_max)^2, the width
of the Wigner spectrum), given as deviations from the window means plus the
two means, it predicts the deviations of the next 64 from those means.  Applied in chunks it extends
a short run of k steps to n_total coefficients, and the continued fraction
(with the usual terminator after that) is evaluated over the extension, so
fewer operator applications are needed for a spectrum close to the long run's.

Training and inference run on the GPU through the library's own kernels
(tdscha_mlp_*: float32 forward / backward and Adam; inference with bfloat16
weights and layer inputs); the plain continued fraction stays the fallback
and the judge: `evaluate` reports both spectral errors against the full run.

    python -m tdscha_gb300.terminator train --out weights.npz
"""
import argparse
import ctypes
import json
import os
import time

import numpy as np

from . import _native as nat

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "data", "terminator_w48_h64.npz")
RY_TO_CM = 109691.40235
WINDOW, HORIZON, HIDDEN = 48, 64, 256

_fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class MLP:
    """The perceptron on the GPU (tdscha_mlp)."""

    def __init__(self, n_in, n_hidden, n_out, seed=0, params=None):
        self.n_in, self.n_h, self.n_out = n_in, n_hidden, n_out
        lib = nat.load()
        h = ctypes.c_void_p()
        nat.check(lib.tdscha_mlp_create(ctypes.byref(h), n_in, n_hidden, n_out))
        self.handle = h
        self.n_par = int(lib.tdscha_mlp_num_params(h))
        if params is None:
            params = self.init_params(seed)
        self.set_params(params)

    def init_params(self, seed):
        """Xavier-uniform weights, zero biases."""
        rng = np.random.default_rng(seed)
        out = []
        for a, b in ((self.n_in, self.n_h), (self.n_h, self.n_h), (self.n_h, self.n_out)):
            lim = np.sqrt(6.0 / (a + b))
            out += [rng.uniform(-lim, lim, (a, b)).ravel(), np.zeros(b)]
        return np.concatenate(out).astype(np.float32)

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.n_par:
            raise ValueError("expected %d parameters, got %d" % (self.n_par, p.size))
        nat.check(nat.load().tdscha_mlp_set_params(self.handle, _fp(p)))

    def get_params(self):
        p = np.empty(self.n_par, dtype=np.float32)
        nat.check(nat.load().tdscha_mlp_get_params(self.handle, _fp(p)))
        return p

    def forward(self, x, bf16=False):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((x.shape[0], self.n_out), dtype=np.float32)
        nat.check(nat.load().tdscha_mlp_forward(self.handle, _fp(x), x.shape[0], int(bool(bf16)),
                                                _fp(y)))
        return y

    def loss_grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        g = np.empty(self.n_par, dtype=np.float32)
        nat.check(nat.load().tdscha_mlp_loss_grad(self.handle, _fp(x), _fp(t), x.shape[0],
                                                  _fp(loss), _fp(g)))
        return float(loss[0]), g

    def train_step(self, xd, td, lr, step, want_loss=False):
        """One Adam step on device tensors (rows x n_in, rows x n_out, float32)."""
        import torch
        loss = np.zeros(1, dtype=np.float32)
        st = torch.cuda.current_stream().cuda_stream
        nat.check(nat.load().tdscha_mlp_train_step(
            self.handle, xd.data_ptr(), td.data_ptr(), xd.shape[0], lr, 0.9, 0.999, 1e-8, step,
            _fp(loss) if want_loss else None, st))
        return float(loss[0]) if want_loss else None

    def close(self):
        if getattr(self, "handle", None):
            nat.load().tdscha_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------- data
def features(a_w, b_w):
    """Network input of one window of normalised coefficients: deviations from
    the window means, then the two means.  Returns (x, mean_a, mean_b)."""
    ma, mb = float(np.mean(a_w)), float(np.mean(b_w))
    return np.concatenate([np.asarray(a_w) - ma, np.asarray(b_w) - mb, [ma, mb]]), ma, mb


def windows(a, b, sigma, k_min=WINDOW, window=WINDOW, horizon=HORIZON, stride=1):
    """(inputs, targets) of every position k in [k_min, n - horizon]: targets
    are the next `horizon` normalised coefficients minus the window means."""
    a = np.asarray(a, dtype=np.float64) / sigma
    b = np.asarray(b, dtype=np.float64) / sigma
    n = min(len(a), len(b))
    xs, ts = [], []
    for k in range(max(k_min, window), n - horizon + 1, stride):
        x, ma, mb = features(a[k - window:k], b[k - window:k])
        xs.append(x)
        ts.append(np.concatenate([a[k:k + horizon] - ma, b[k:k + horizon] - mb]))
    if not xs:
        return np.zeros((0, 2 * window + 2)), np.zeros((0, 2 * horizon))
    return np.array(xs), np.array(ts)


def generate_runs(n_runs, n_steps, seed=0, m_range=(48, 160), n_configs=4000, batch=20,
                  anh_range=(0.01, 0.1), precision="mixed", reorth=True, verbose=False):
    """Coefficient sequences of symmetric Wigner Lanczos runs on seeded
    synthetic ensembles: M log-uniform in m_range, N = n_configs, the cubic /
    quartic force scale uniform in anh_range; random unit R1 start; full
    re-orthogonalisation, or (reorth=False) the reference's default
    recurrence, whose cost per step does not grow with the step index.
    Returns [(a, b, sigma, M)]."""
    from .batch import run_batch
    from .DynamicalLanczos import Lanczos
    from .synthetic import make_ensemble, random_R1
    rng = np.random.default_rng(seed)
    out = []
    for b0 in range(0, n_runs, batch):
        runs = []
        for i in range(b0, min(n_runs, b0 + batch)):
            M = int(np.exp(rng.uniform(np.log(m_range[0]), np.log(m_range[1]))))
            anh = float(rng.uniform(*anh_range))
            e = make_ensemble(M, n_configs, seed=int(rng.integers(1 << 30)), anh_scale=anh,
                              rho_sigma=0.1)
            lz = Lanczos.from_arrays(e["X"], e["Y"], e["w"], e["rho"], e["T"], use_wigner=True,
                                     precision=precision)
            lz.init(use_symmetries=False)
            lz.full_reorth = bool(reorth)
            lz.prepare_perturbation(random_R1(M, int(rng.integers(1 << 30))), masses_exp=0)
            runs.append(lz)
        run_batch(runs, n_steps)
        for lz in runs:
            sigma = float((2 * np.max(lz.w)) ** 2)
            out.append((np.array(lz.a_coeffs), np.array(lz.b_coeffs), sigma, lz.n_modes))
            lz._invalidate()
        if verbose:
            print("generated %d / %d runs" % (len(out), n_runs))
    return out


def train(runs, iters=3000, batch=512, lr=1e-3, seed=0, k_min=WINDOW, verbose=False):
    """Fit the perceptron on every window of the given runs (GPU); returns
    (MLP, loss history)."""
    import torch
    X, T = [], []
    for a, b, sigma, _ in runs:
        x, t = windows(a, b, sigma, k_min=k_min)
        X.append(x)
        T.append(t)
    X = torch.from_numpy(np.concatenate(X).astype(np.float32)).cuda()
    T = torch.from_numpy(np.concatenate(T).astype(np.float32)).cuda()
    mlp = MLP(2 * WINDOW + 2, HIDDEN, 2 * HORIZON, seed=seed)
    g = torch.Generator(device="cuda").manual_seed(seed)
    hist = []
    for it in range(1, iters + 1):
        idx = torch.randint(0, X.shape[0], (batch,), device="cuda", generator=g)
        xb, tb = X[idx].contiguous(), T[idx].contiguous()
        # cosine decay of the step size
        lr_it = lr * 0.5 * (1 + np.cos(np.pi * (it - 1) / iters))
        loss = mlp.train_step(xb, tb, lr_it, it, want_loss=(it % 100 == 0 or it == 1))
        if loss is not None:
            hist.append((it, loss))
            if verbose:
                print("iter %d loss %.3e" % (it, loss))
    return mlp, hist


# ---------------------------------------------------------------- inference
class LearnedTerminator:
    """Extends measured Lanczos coefficients with the network's prediction."""

    def __init__(self, params=None, window=WINDOW, horizon=HORIZON, hidden=HIDDEN):
        self.window, self.horizon, self.hidden = window, horizon, hidden
        if params is None:
            if not os.path.exists(DEFAULT_WEIGHTS):
                raise IOError("no trained weights at %s (python -m tdscha_gb300.terminator train)"
                              % DEFAULT_WEIGHTS)
            params = np.load(DEFAULT_WEIGHTS)["params"]
        self.mlp = MLP(2 * window + 2, hidden, 2 * horizon, params=params)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        return cls(d["params"], int(d["window"]), int(d["horizon"]), int(d["hidden"]))

    def save(self, path, **extra):
        np.savez_compressed(path, params=self.mlp.get_params(), window=self.window,
                            horizon=self.horizon, hidden=self.hidden, **extra)

    def extend(self, a, b, sigma, n_total, bf16=True):
        """a, b continued to n_total coefficients (chunks of `horizon`)."""
        a = list(np.asarray(a, dtype=np.float64) / sigma)
        b = list(np.asarray(b, dtype=np.float64) / sigma)
        n = min(len(a), len(b))
        a, b = a[:n], b[:n]
        if n < self.window:
            raise ValueError("need at least %d coefficients" % self.window)
        while len(a) < n_total:
            x, ma, mb = features(a[-self.window:], b[-self.window:])
            y = self.mlp.forward(x[None, :], bf16=bf16)[0].astype(np.float64)
            a += list(y[:self.horizon] + ma)
            b += list(np.maximum(y[self.horizon:] + mb, 0.0))   # b_n >= 0 by construction
        return np.array(a[:n_total]) * sigma, np.array(b[:n_total]) * sigma

    def green_function(self, lanczos, w_array, n_total, smearing=0.0, use_terminator=True,
                       last_average=1):
        """G(w) of a symmetric Wigner run extended to n_total coefficients."""
        sigma = float((2 * np.max(lanczos.w)) ** 2)
        a, b = self.extend(lanczos.a_coeffs, lanczos.b_coeffs, sigma, n_total)
        return continued_fraction(a, b, w_array, smearing, lanczos.perturbation_modulus,
                                  use_terminator, last_average)


def continued_fraction(a, b, w_array, smearing=0.0, modulus=1.0, use_terminator=True,
                       last_average=1, use_wigner=True):
    """G(w) on the GPU (tdscha_continued_fraction) with c = b."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b[:len(a) - 1] if len(b) >= len(a) else b, dtype=np.float64)
    w = np.ascontiguousarray(w_array, dtype=np.float64)
    out = np.zeros(2 * w.size)
    nat.check(nat.load().tdscha_continued_fraction(
        nat.dp(a), len(a), nat.dp(b), len(b), nat.dp(b), len(b), nat.dp(w.ravel()), w.size,
        1 if use_wigner else 0, float(modulus), 0, 0.0, 1 if use_terminator else 0,
        int(last_average), float(smearing), 0, nat.dp(out)))
    return out[0::2] + 1j * out[1::2]


def spectral_error(g, g_ref):
    A, R = -np.imag(g), -np.imag(g_ref)
    return float(np.linalg.norm(A - R) / np.linalg.norm(R))


def evaluate(term, runs, k, n_total, n_w=2000, w_max_cm=1100.0, smearing_cm=5.0,
             k_grid=None):
    """Spectral errors against each run's full n_total-step spectrum (2000
    points, 5 cm^-1 smearing, square-root terminator): the first k steps with
    the standard terminator, and the first k steps extended by the network to
    n_total.  `saved_applications` is, per run, how many more steps the plain
    method needs (every step count from k on, unless k_grid says otherwise)
    to be as close to the full spectrum as the extended k-step run (0 when it
    never is worse)."""
    w = np.linspace(0, w_max_cm, n_w) / RY_TO_CM
    sm = smearing_cm / RY_TO_CM
    every = k_grid is None
    k_grid = list(range(k, n_total + 1)) if k_grid is None else k_grid
    plain, learned, saved = [], [], []
    for a, b, sigma, _ in runs:
        g_ref = continued_fraction(a[:n_total], b[:n_total], w, sm)
        errs = {kk: spectral_error(continued_fraction(a[:kk], b[:kk], w, sm), g_ref) for kk in k_grid}
        ae, be = term.extend(a[:k], b[:k], sigma, n_total)
        el = spectral_error(continued_fraction(ae, be, w, sm), g_ref)
        plain.append(errs[k])
        learned.append(el)
        need = next((kk for kk in k_grid if errs[kk] <= el), n_total)
        saved.append(max(0, need - k))
    return {"k": k, "n_total": n_total, "runs": len(runs),
            "step_grid": "every step" if every else "%d points" % len(k_grid),
            "plain_terminator_err_median": float(np.median(plain)),
            "learned_err_median": float(np.median(learned)),
            "plain_terminator_err_mean": float(np.mean(plain)),
            "learned_err_mean": float(np.mean(learned)),
            "learned_better_fraction": float(np.mean(np.array(learned) < np.array(plain))),
            "saved_applications_median": float(np.median(saved)),
            "saved_applications_mean": float(np.mean(saved))}


def save_runs(path, **sets):
    """Coefficient sequences of run sets in one npz: per set, a and b padded
    with NaN to the longest run, sigma and M."""
    out = {}
    for name, runs in sets.items():
        n = max(len(a) for a, _, _, _ in runs)
        A = np.full((len(runs), n), np.nan)
        B = np.full((len(runs), n), np.nan)
        for i, (a, b, _, _) in enumerate(runs):
            A[i, :len(a)] = a
            B[i, :len(b)] = b
        out[name + "_a"], out[name + "_b"] = A, B
        out[name + "_sigma"] = np.array([r[2] for r in runs])
        out[name + "_M"] = np.array([r[3] for r in runs])
    np.savez_compressed(path, **out)


def load_runs(path, name):
    d = np.load(path)
    runs = []
    for a, b, s, m in zip(d[name + "_a"], d[name + "_b"], d[name + "_sigma"], d[name + "_M"]):
        runs.append((a[~np.isnan(a)], b[~np.isnan(b)], float(s), int(m)))
    return runs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "generate"])
    ap.add_argument("--data", default=None,
                    help="train: read the runs from this file (written by generate)")
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--n-train", type=int, default=200)
    ap.add_argument("--n-test", type=int, default=20)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--k", type=int, default=100)
    ap.add_argument("--iters", type=int, default=20000)
    ap.add_argument("--m-range", type=int, nargs=2, default=(96, 384))
    ap.add_argument("--n-configs", type=int, default=20000)
    ap.add_argument("--train-precision", default="fp64", choices=["mixed", "fp64"])
    ap.add_argument("--test-precision", default="fp64", choices=["mixed", "fp64"])
    ap.add_argument("--batch", type=int, default=20)
    ap.add_argument("--reorth", action="store_true",
                    help="full re-orthogonalisation in the generated runs (its cost grows "
                         "with the step index; off: the reference's default recurrence)")
    ap.add_argument("--report", default=None)
    args = ap.parse_args()
    t0 = time.time()
    gen = dict(m_range=tuple(args.m_range), n_configs=args.n_configs, batch=args.batch,
               reorth=args.reorth)
    if args.data and args.cmd == "train":
        train_runs, test_runs = load_runs(args.data, "train"), load_runs(args.data, "test")
        t_tr = t1 = time.time()
    else:
        train_runs = generate_runs(args.n_train, args.steps, seed=1,
                                   precision=args.train_precision, verbose=True, **gen)
        t_tr = time.time()
        test_runs = generate_runs(args.n_test, args.steps, seed=2,
                                  precision=args.test_precision, verbose=True, **gen)
        t1 = time.time()
    if args.cmd == "generate":
        save_runs(args.out, train=train_runs, test=test_runs)
        print(json.dumps({"saved": args.out, "train": len(train_runs), "test": len(test_runs),
                          "seconds": t1 - t0}))
        return
    mlp, hist = train(train_runs, iters=args.iters)
    t2 = time.time()
    term = LearnedTerminator(mlp.get_params())
    rep = evaluate(term, test_runs, args.k, args.steps)
    rep.update(train_runs=args.n_train, steps=args.steps, data_s=t1 - t0,
               train_data_s=t_tr - t0, train_s=t2 - t1, loss_first=hist[0][1],
               loss_last=hist[-1][1], iters=args.iters, m_range=list(args.m_range),
               n_configs=args.n_configs, train_precision=args.train_precision,
               test_precision=args.test_precision, reorth=bool(args.reorth))
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    term.save(args.out, report=json.dumps(rep))
    print(json.dumps(rep))
    if args.report:
        with open(args.report, "w") as fp:
            json.dump({"report": rep, "loss_history": hist}, fp)


if __name__ == "__main__":
    main()

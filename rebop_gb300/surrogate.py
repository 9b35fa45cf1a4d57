"""Learned surrogate of the dimerization ensemble (the dimer network, its 5
rate constants log-uniform over one decade either side of their values, t in
[0, 1]).

A query (u, t) -- the log10 factors u of the five rate constants and the time
-- gets the count distributions of protein and dimer.  Their deterministic
part comes from the network's reaction rate equations (the SSA's mean-field
limit), integrated per query on the GPU (rbg_mdn_rre): b = log(x_RRE + 1).  A
multilayer perceptron (8 inputs: u, t, b -> 4 x 256 SiLU -> 112) maps the query
to a count-aware head per species: a categorical over the counts 0 .. 30 and a
tail class, and for the tail an 8-component Gaussian mixture over the residual
log(n + v) - b (v ~ U[0, 1) dequantises the integer n); a tail draw z becomes
the count floor(exp(z + b)).  Small counts are thus exact classes -- early in a
trajectory the dimer count is 0, 1 or 2 -- and for large ones the network
learns only the stochastic correction around the rate equations, a small and
smooth function that BF16 resolves finely.  The two species' draws are
independent: the head models each marginal distribution, not their
correlation.  (head="mixture" selects an 8-component diagonal Gaussian
mixture over both residuals jointly instead.)  Weights are BF16 with FP32 master copies; every
forward and backward GEMM runs on the 5th-generation tensor cores (tcgen05.mma
into tensor memory, FP32 accumulation; the forward products with operands
loaded by TMA), inference runs the whole network in one fused tcgen05 kernel
(MDN.infer), and the rate-equation solver, the loss, its gradient, the
optimiser and the sampler are the engine's own kernels (rebop_gb300/csrc/mdn.cu).  PyTorch only holds the device memory.  Training
data, the validation that decides where the surrogate is trusted, and the
fallback for the rest all come from the SSA engine itself.
"""

from __future__ import annotations

import numpy as np

from ._lib import check, lib

RATES0 = (25.0, 1000.0, 0.001, 0.1, 1.0)  # G->G+M, M->M+P, 2P->D, M->0, P->0
X0 = (1, 0, 0, 0)
EXPS = ([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 2, 0], [0, 1, 0, 0], [0, 0, 1, 0])
DIFFS = ([0, 1, 0, 0], [0, 0, 1, 0], [0, 0, -2, 1], [0, -1, 0, 0], [0, 0, -1, 0])
N_QUERY, N_IN, HIDDEN, LAYERS, K = 6, 8, 256, 4, 8
NC, KT = 32, 8                # count classes (0 .. 30 and the tail), tail components
N_OUT_MIX = 5 * K
RRE_STEPS = 128


def dimer_network(rates=RATES0):
    from .api import Network, Rate

    net = Network(4)
    for k, e, d in zip(rates, EXPS, DIFFS):
        net.add_reaction(Rate.lma(k, e), d)
    return net


_RRE_CONST: dict = {}


def _rre_constants(device):
    """The rate equations' constant tensors on `device`, made once: a copy from
    pageable host memory waits for the stream, which would serialise every
    query batch with the previous one's kernels."""
    import torch

    key = str(device)
    if key not in _RRE_CONST:
        _RRE_CONST[key] = (torch.tensor(RATES0, dtype=torch.float32, device=device),
                           torch.tensor(EXPS, dtype=torch.int32, device=device),
                           torch.tensor(DIFFS, dtype=torch.float32, device=device),
                           torch.tensor(X0, dtype=torch.float32, device=device),
                           torch.tensor([2, 3], dtype=torch.int32, device=device))
    return _RRE_CONST[key]


def rre_log_means(x):
    """b = log(x_RRE + 1) of (protein, dimer) at each query row of x [Q][6]
    (u, t) on the GPU: the reaction rate equations integrated from the initial
    counts to t (rbg_mdn_rre, RK4 in float32, RRE_STEPS steps)."""
    import torch

    x = x.to("cuda", torch.float32).contiguous()
    Q = x.shape[0]
    r0, E, N, x0, idx = _rre_constants(x.device)
    rates = (r0 * torch.pow(10.0, x[:, :5])).contiguous()
    t = x[:, 5].contiguous()
    out = torch.empty(Q, 2, dtype=torch.float32, device=x.device)
    check(lib.rbg_mdn_rre(rates.data_ptr(), t.data_ptr(), Q, 4, 5, E.data_ptr(), N.data_ptr(), x0.data_ptr(),
                          RRE_STEPS, idx.data_ptr(), 2, out.data_ptr(), torch.cuda.current_stream().cuda_stream))
    return torch.log1p(out)


def features(x):
    """Network inputs of queries x [Q][6]: (u, t, b)."""
    import torch

    x = x.to("cuda", torch.float32).contiguous()
    return torch.cat([x, rre_log_means(x)], dim=1).contiguous()


def generate(n_traj: int, seed: int, nb_steps: int = 100, net=None, per_traj: int = 1, chunk: int = 1 << 17,
             draws: int = 1):
    """SSA training data: rate factors 10^u, u ~ U[-1, 1]^5, and a sample time
    from the grid t = i / nb_steps per tuple; each tuple gets `draws`
    trajectories (1: every tuple an independent draw of its distribution) and
    each trajectory `per_traj` sample times.  Returns queries [n][6] (u, t),
    targets [n][4] (the counts n of protein and dimer, then the residuals
    log(n + v) - b, v ~ U[0, 1)) and b [n][2]."""
    import torch

    rng = np.random.default_rng(seed)
    net = net or dimer_network()
    xs, ys = [], []
    for c0 in range(0, n_traj, chunk):
        n = min(chunk, n_traj - c0)
        n_u = -(-n // draws)
        u = np.repeat(rng.uniform(-1.0, 1.0, size=(n_u, 5)), draws, axis=0)[:n]
        rates = np.asarray(RATES0) * 10.0 ** u
        seeds = rng.integers(np.iinfo(np.uint64).max, size=n, dtype=np.uint64)
        res = net.run_ensemble(list(X0), seeds, 1.0, nb_steps, save=[2, 3], rates=rates, want_events=False)
        c = res.counts  # [nb+1][2][n]
        ti = np.repeat(rng.integers(0, nb_steps + 1, size=(n_u, per_traj)), draws, axis=0)[:n]
        j = np.repeat(np.arange(n), per_traj)
        t = ti.reshape(-1)
        xs.append(np.concatenate([u[j], (t / nb_steps)[:, None]], axis=1))
        cnt = np.stack([c[t, 0, j], c[t, 1, j]], axis=1).astype(np.float64)
        ys.append((cnt, np.log(cnt + rng.uniform(0.0, 1.0, size=cnt.shape))))
    x = np.concatenate(xs).astype(np.float32)
    b = rre_log_means(torch.from_numpy(x)).cpu().numpy().astype(np.float64)
    cnt = np.concatenate([a for a, _ in ys])
    y = np.concatenate([cnt, np.concatenate([r for _, r in ys]) - b], axis=1).astype(np.float32)
    return x, y, b.astype(np.float32)


class MDN:
    """The surrogate network; see the module docstring."""

    def __init__(self, seed: int = 0, device: str = "cuda", head: str = "count", tail: int = KT):
        import torch

        if head not in ("count", "mixture"):
            raise ValueError("head must be 'count' or 'mixture'")
        self.torch = torch
        self.dev = device
        self.head = head
        self.tail = int(tail)
        self.n_out = 2 * (NC + 3 * self.tail) if head == "count" else N_OUT_MIX
        g = torch.Generator().manual_seed(seed)
        dims = [N_IN] + [HIDDEN] * LAYERS + [self.n_out]
        self.W, self.b = [], []
        for i in range(len(dims) - 1):
            fan_in, fan_out = dims[i], dims[i + 1]
            w = torch.randn(fan_out, fan_in, generator=g, dtype=torch.float32) * (1.0 / fan_in) ** 0.5
            self.W.append(w.to(device))
            self.b.append(torch.zeros(fan_out, dtype=torch.float32, device=device))
        self.Wb = [w.to(torch.bfloat16) for w in self.W]
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.step = 0
        import os

        self.use_tc05 = os.environ.get("RB_GEMM", "tc05") != "mma"
        self.tc_err = torch.zeros(1, dtype=torch.int32, device=device)
        # input and target normalisation (set from the training data)
        self.x_mean = torch.zeros(N_IN, device=device)
        self.x_std = torch.ones(N_IN, device=device)

    # ---------------------------------------------------------------- kernels
    def _s(self):
        return self.torch.cuda.current_stream().cuda_stream

    def _gemm(self, A, ta, B, tb, C, M, N, K_, lda, ldb, beta=0.0):
        # tcgen05 with tensor-memory accumulators; RB_GEMM=mma selects the
        # mma.sync kernel instead
        if self.use_tc05:
            check(lib.rbg_mdn_gemm_tc05(A.data_ptr(), lda, int(ta), B.data_ptr(), ldb, int(tb), C.data_ptr(), N, M,
                                        N, K_, float(beta), self.tc_err.data_ptr(), self._s()))
        else:
            check(lib.rbg_mdn_gemm(A.data_ptr(), lda, int(ta), B.data_ptr(), ldb, int(tb), C.data_ptr(), N, M, N,
                                   K_, float(beta), self._s()))

    def check_errors(self):
        """Raise if a tensor-core completion wait ran out since construction."""
        if self.use_tc05 and int(self.tc_err.item()):
            raise RuntimeError("tcgen05 GEMM: a completion wait ran out")

    def forward(self, x):
        """x [B][8] float features (unnormalised u, t, b) -> head outputs [B][n_out];
        keeps the activations for backward."""
        torch = self.torch
        B = x.shape[0]
        h = ((x - self.x_mean) / self.x_std).to(torch.bfloat16).contiguous()
        self._H, self._Z = [h], []
        for i, (Wb, b) in enumerate(zip(self.Wb, self.b)):
            out = Wb.shape[0]
            z = torch.empty(B, out, dtype=torch.float32, device=self.dev)
            self._gemm(h, False, Wb, True, z, B, out, Wb.shape[1], h.shape[1], Wb.shape[1])
            last = i == len(self.Wb) - 1
            hn = None if last else torch.empty(B, out, dtype=torch.bfloat16, device=self.dev)
            check(lib.rbg_mdn_bias_act(z.data_ptr(), b.data_ptr(), hn.data_ptr() if hn is not None else None, B,
                                       out, 0 if last else 1, self._s()))
            self._Z.append(z)
            if not last:
                self._H.append(hn)
                h = hn
        return self._Z[-1]

    def loss_and_grad(self, x, y):
        """Mean negative log-likelihood and the gradients (dW, db) of every layer."""
        torch = self.torch
        B = x.shape[0]
        o = self.forward(x)
        loss = torch.empty(B, dtype=torch.float32, device=self.dev)
        G = torch.empty_like(o)
        if self.head == "count":
            check(lib.rbg_mdn_count_loss(o.data_ptr(), y.data_ptr(), B, self.tail, loss.data_ptr(), G.data_ptr(),
                                         self._s()))
        else:
            yr = y[:, 2:].contiguous()
            check(lib.rbg_mdn_loss(o.data_ptr(), yr.data_ptr(), B, K, loss.data_ptr(), G.data_ptr(), self._s()))
        dW = [None] * len(self.W)
        db = [None] * len(self.W)
        n = len(self.W)
        # head: bias gradient and a BF16 copy of dO
        d = torch.empty(B, self.n_out, dtype=torch.bfloat16, device=self.dev)
        db[n - 1] = torch.empty(self.n_out, dtype=torch.float32, device=self.dev)
        check(lib.rbg_mdn_head_backward(G.data_ptr(), d.data_ptr(), db[n - 1].data_ptr(), B, self.n_out,
                                        self._s()))
        for i in range(n - 1, -1, -1):
            out, inp = self.W[i].shape
            h = self._H[i]
            dW[i] = torch.empty(out, inp, dtype=torch.float32, device=self.dev)
            # dW = d^T h: op(A) = d^T (A = d [B][out]), op(B) = h [B][inp]
            self._gemm(d, True, h, False, dW[i], out, inp, B, out, inp)
            if i == 0:
                break
            dh = torch.empty(B, inp, dtype=torch.float32, device=self.dev)
            # dh = d W: op(A) = d [B][out], op(B) = W [out][inp]
            self._gemm(d, False, self.Wb[i], False, dh, B, inp, out, out, inp)
            dz = torch.empty(B, inp, dtype=torch.bfloat16, device=self.dev)
            db[i - 1] = torch.empty(inp, dtype=torch.float32, device=self.dev)
            check(lib.rbg_mdn_silu_backward(self._Z[i - 1].data_ptr(), dh.data_ptr(), dz.data_ptr(),
                                            db[i - 1].data_ptr(), B, inp, self._s()))
            d = dz
        return loss.mean(), dW, db

    def train_step(self, x, y, lr: float):
        loss, dW, db = self.loss_and_grad(x, y)
        self.step += 1
        for i in range(len(self.W)):
            check(lib.rbg_mdn_adam(self.W[i].data_ptr(), self.Wb[i].data_ptr(), dW[i].data_ptr(),
                                   self.mW[i].data_ptr(), self.vW[i].data_ptr(), self.W[i].numel(), lr, 0.9, 0.999,
                                   1e-8, self.step, self._s()))
            check(lib.rbg_mdn_adam(self.b[i].data_ptr(), None, db[i].data_ptr(), self.mb[i].data_ptr(),
                                   self.vb[i].data_ptr(), self.b[i].numel(), lr, 0.9, 0.999, 1e-8, self.step,
                                   self._s()))
        return loss

    def fit(self, x, y, epochs: int = 20, batch: int = 4096, lr: float = 2e-3, seed: int = 0, log=None):
        """Train on host arrays x [N][6] (queries u, t), y [N][4] (counts, residuals)."""
        torch = self.torch
        X = features(torch.from_numpy(np.ascontiguousarray(x)))
        Y = torch.from_numpy(np.ascontiguousarray(y)).to(self.dev)
        self.x_mean = X.mean(0)
        self.x_std = X.std(0) + 1e-6
        n = X.shape[0]
        g = torch.Generator(device=self.dev).manual_seed(seed)
        steps = epochs * (n // batch)
        k = 0
        for ep in range(epochs):
            perm = torch.randperm(n, generator=g, device=self.dev)
            tot, cnt = 0.0, 0
            for s in range(n // batch):
                idx = perm[s * batch:(s + 1) * batch]
                lr_k = lr * 0.5 * (1.0 + np.cos(np.pi * k / steps))  # cosine decay
                loss = self.train_step(X[idx].contiguous(), Y[idx].contiguous(), lr_k)
                if s % 50 == 0:
                    tot, cnt = tot + float(loss), cnt + 1
                k += 1
            if log:
                log(f"epoch {ep}: loss {tot / max(cnt, 1):.4f}")
        self.check_errors()

    def infer(self, F):
        """Head outputs [Q][n_out] for feature rows F [Q][8] (unnormalised), by the
        fused inference kernel: the whole MLP in one launch, activations kept
        in shared memory (``rbg_mdn_infer``).  Falls back to the layer-by-layer
        forward pass for heads it does not cover (n_out not a multiple of 4) or
        with RB_GEMM=mma."""
        torch = self.torch
        F = F.contiguous()
        if not self.use_tc05 or self.n_out % 4 != 0 or self.n_out > HIDDEN or LAYERS != 4 or HIDDEN != 256:
            return self.forward(F)
        O = torch.empty(F.shape[0], self.n_out, dtype=torch.float32, device=self.dev)
        W, b = self.Wb, self.b
        check(lib.rbg_mdn_infer(F.data_ptr(), F.shape[0], F.shape[1], self.x_mean.data_ptr(), self.x_std.data_ptr(),
                                W[0].data_ptr(), W[1].data_ptr(), W[2].data_ptr(), W[3].data_ptr(), W[4].data_ptr(),
                                b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr(), b[3].data_ptr(), b[4].data_ptr(),
                                self.n_out, O.data_ptr(), self.tc_err.data_ptr(), self._s()))
        return O

    def sample_counts(self, x, n_draws: int, seed: int = 1):
        """n_draws samples of (protein, dimer) counts at each query row of x [Q][6]:
        the rate equations and one forward pass per query, then n_draws draws
        from its head, each turned into a count by the sampler kernel."""
        F = features(self._queries(x))
        torch = self.torch
        o = self.infer(F)
        base = F[:, N_QUERY:].contiguous()
        c = torch.empty(F.shape[0] * n_draws, 2, dtype=torch.float32, device=self.dev)
        if self.head == "count":
            work = torch.empty_like(o)  # the prepared per-query distributions
            check(lib.rbg_mdn_count_sample(o.data_ptr(), c.shape[0], self.tail, int(seed), c.data_ptr(), int(n_draws),
                                           base.data_ptr(), work.data_ptr(), self._s()))
        else:
            check(lib.rbg_mdn_sample(o.data_ptr(), c.shape[0], K, int(seed), c.data_ptr(), int(n_draws),
                                     base.data_ptr(), self._s()))
        return c.view(F.shape[0], n_draws, 2)

    def predict_params(self, x):
        """Head outputs at each query row (one forward pass): [Q][n_out]."""
        return self.infer(features(self._queries(x)))

    def _queries(self, x):
        torch = self.torch
        if isinstance(x, torch.Tensor):
            return x.to(self.dev, torch.float32).contiguous()
        return torch.as_tensor(np.ascontiguousarray(x, dtype=np.float32), device=self.dev)


class Surrogate:
    """A trained MDN plus the validation that says where it may answer.

    `validate` compares the MDN with fresh SSA batches at held-out points; a
    query then takes the MDN's answer when the nearest validation point (in
    (u, t) space) met the tolerance, and falls back to the SSA engine
    otherwise."""

    def __init__(self, model: MDN, tol: float = 0.01):
        self.model = model
        self.tol = tol
        self.points = None
        self.ok = None

    def validate(self, n_points: int, n_ssa: int, seed: int, net=None, model_draws: int | None = None):
        """Per held-out point: relative W1 and KS of the MDN against a fresh SSA
        batch of n_ssa trajectories, and the same for a second independent SSA
        batch (the sampling-noise floor of the comparison).  The MDN's side is
        `model_draws` draws (default 10 n_ssa: the surrogate draws cheaply, so
        its own sampling noise stays small next to the SSA batch's)."""
        rng = np.random.default_rng(seed)
        u = rng.uniform(-1, 1, size=(n_points, 5))
        ti = rng.integers(1, 101, size=n_points)
        t = ti / 100.0
        net = net or dimer_network()
        rates = np.repeat(np.asarray(RATES0) * 10.0 ** u, n_ssa, axis=0)
        runs = []
        import time

        for rep in range(2):
            seeds = rng.integers(np.iinfo(np.uint64).max, size=n_points * n_ssa, dtype=np.uint64)
            t0 = time.perf_counter()
            res = net.run_ensemble(list(X0), seeds, 1.0, 100, save=[2, 3], rates=rates, want_events=False)
            runs.append((res.counts, time.perf_counter() - t0, res.stats["kernel_ms"]))
        x = np.concatenate([u, t[:, None]], axis=1).astype(np.float32)
        md = model_draws or 10 * n_ssa
        draws = np.concatenate([self.model.sample_counts(x[k:k + 16], md, seed=seed + 1 + k).cpu().numpy()
                                for k in range(0, n_points, 16)])
        out = {"w1": np.zeros((n_points, 2)), "ks": np.zeros((n_points, 2)), "w1_floor": np.zeros((n_points, 2)),
               "mean": np.zeros((n_points, 2)), "t": t, "model_draws": md}
        for p in range(n_points):
            sl = slice(p * n_ssa, (p + 1) * n_ssa)
            for s in range(2):
                a = runs[0][0][ti[p], s, sl].astype(np.float64)
                b = runs[1][0][ti[p], s, sl].astype(np.float64)
                m = draws[p, :, s]
                mean = max(a.mean(), 1.0)
                out["mean"][p, s] = a.mean()
                out["w1"][p, s] = wasserstein1(m, a) / mean
                out["w1_floor"][p, s] = wasserstein1(b, a) / mean
                out["ks"][p, s] = ks_distance(m, a)
        self.points = x
        self.features = features(torch_tensor(x)).cpu().numpy()
        self.ok = (out["w1"] <= self.tol).all(axis=1)
        out["ssa_seconds"] = runs[0][1]
        out["ssa_kernel_ms"] = runs[0][2]
        return out

    def answer(self, x):
        """Which queries of x [Q][6] the MDN answers (True) and which fall back:
        a query takes the verdict of the nearest validation point in (t, b) --
        the time and the rate-equation log counts, which set how the count
        distributions look -- scaled to unit spread."""
        f = features(torch_tensor(np.asarray(x, dtype=np.float32))).cpu().numpy()[:, N_QUERY - 1:]
        ref = self.features[:, N_QUERY - 1:]
        scale = ref.std(0) + 1e-6
        ok = np.empty(len(f), dtype=bool)
        for k in range(0, len(f), 4096):
            d = (((f[k:k + 4096, None, :] - ref[None, :, :]) / scale) ** 2).sum(-1)
            ok[k:k + 4096] = self.ok[np.argmin(d, axis=1)]
        return ok


def torch_tensor(x):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32))


def wasserstein1(a: np.ndarray, b: np.ndarray) -> float:
    """W1 distance of two empirical samples: the integral of |F_a - F_b|."""
    a, b = np.sort(a), np.sort(b)
    if len(a) == len(b):
        return float(np.mean(np.abs(a - b)))
    grid = np.union1d(a, b)
    fa = np.searchsorted(a, grid[:-1], side="right") / len(a)
    fb = np.searchsorted(b, grid[:-1], side="right") / len(b)
    return float(np.sum(np.abs(fa - fb) * np.diff(grid)))


def ks_distance(a: np.ndarray, b: np.ndarray) -> float:
    grid = np.union1d(a, b)
    fa = np.searchsorted(np.sort(a), grid, side="right") / len(a)
    fb = np.searchsorted(np.sort(b), grid, side="right") / len(b)
    return float(np.max(np.abs(fa - fb)))

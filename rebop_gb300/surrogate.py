"""Learned surrogate of the dimerization ensemble (configs: dimer network,
5 rate constants log-uniform over one decade either side of their values, t
in [0, 1]).

A multilayer perceptron (6 inputs -> 4 x 256 SiLU -> 40) maps
(log10 rate factors, t) to an 8-component diagonal Gaussian mixture over
(log1p protein, log1p dimer) counts.  Weights are BF16 with FP32 master
copies; every forward and backward GEMM runs in the engine's tensor-core
kernel with FP32 accumulation, and the loss, its gradient, the optimiser and
the sampler are the engine's own kernels (rebop_gb300/csrc/mdn.cu).  PyTorch
only holds the device memory.  Training data, the validation that decides
where the surrogate is trusted, and the fallback for the rest all come from
the SSA engine itself.
"""

from __future__ import annotations

import numpy as np

from ._lib import check, lib

RATES0 = (25.0, 1000.0, 0.001, 0.1, 1.0)  # G->G+M, M->M+P, 2P->D, M->0, P->0
X0 = (1, 0, 0, 0)
N_IN, HIDDEN, LAYERS, K = 6, 256, 4, 8
N_OUT = 5 * K


def dimer_network(rates=RATES0):
    from .api import Network, Rate

    net = Network(4)
    for k, e, d in zip(rates, ([1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 2, 0], [0, 1, 0, 0], [0, 0, 1, 0]),
                       ([0, 1, 0, 0], [0, 0, 1, 0], [0, 0, -2, 1], [0, -1, 0, 0], [0, 0, -1, 0])):
        net.add_reaction(Rate.lma(k, e), d)
    return net


def generate(n_traj: int, seed: int, nb_steps: int = 100, net=None):
    """SSA training data: per-trajectory rate factors 10^u, u ~ U[-1, 1]^5, and
    every trajectory's samples at t = i / nb_steps.  Returns inputs [n*(nb+1)][6]
    (u, t), targets [n*(nb+1)][2] (log1p protein, log1p dimer) and the raw counts."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1.0, 1.0, size=(n_traj, 5))
    rates = np.asarray(RATES0) * 10.0 ** u
    seeds = rng.integers(np.iinfo(np.uint64).max, size=n_traj, dtype=np.uint64)
    net = net or dimer_network()
    res = net.run_ensemble(list(X0), seeds, 1.0, nb_steps, save=[2, 3], rates=rates, want_events=False)
    c = res.counts  # [nb+1][2][n]
    t = np.arange(nb_steps + 1) / nb_steps
    x = np.concatenate([np.repeat(u[None], nb_steps + 1, 0), np.broadcast_to(t[:, None, None], (nb_steps + 1, n_traj, 1))],
                       axis=2).reshape(-1, 6)
    y = np.log1p(np.transpose(c, (0, 2, 1)).reshape(-1, 2).astype(np.float64))
    return x.astype(np.float32), y.astype(np.float32), c


class MDN:
    """The surrogate network; see the module docstring."""

    def __init__(self, seed: int = 0, device: str = "cuda"):
        import torch

        self.torch = torch
        self.dev = device
        g = torch.Generator().manual_seed(seed)
        dims = [N_IN] + [HIDDEN] * LAYERS + [N_OUT]
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
        # input and target normalisation (set from the training data)
        self.x_mean = torch.zeros(N_IN, device=device)
        self.x_std = torch.ones(N_IN, device=device)

    # ---------------------------------------------------------------- kernels
    def _s(self):
        return self.torch.cuda.current_stream().cuda_stream

    def _gemm(self, A, ta, B, tb, C, M, N, K_, lda, ldb, beta=0.0):
        check(lib.rbg_mdn_gemm(A.data_ptr(), lda, int(ta), B.data_ptr(), ldb, int(tb), C.data_ptr(), N, M, N, K_,
                               float(beta), self._s()))

    def forward(self, x):
        """x [B][6] float (unnormalised u, t) -> head outputs [B][40]; keeps the
        activations for backward."""
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
        check(lib.rbg_mdn_loss(o.data_ptr(), y.data_ptr(), B, K, loss.data_ptr(), G.data_ptr(), self._s()))
        dW = [None] * len(self.W)
        db = [None] * len(self.W)
        n = len(self.W)
        # head: bias gradient and a BF16 copy of dO
        d = torch.empty(B, N_OUT, dtype=torch.bfloat16, device=self.dev)
        db[n - 1] = torch.empty(N_OUT, dtype=torch.float32, device=self.dev)
        check(lib.rbg_mdn_head_backward(G.data_ptr(), d.data_ptr(), db[n - 1].data_ptr(), B, N_OUT, self._s()))
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
        """Train on host arrays x [N][6], y [N][2] (log1p counts)."""
        torch = self.torch
        X = torch.from_numpy(np.ascontiguousarray(x)).to(self.dev)
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

    def sample_counts(self, x, n_draws: int, seed: int = 1):
        """n_draws samples of (protein, dimer) counts at each query row of x [Q][6]."""
        torch = self.torch
        X = torch.as_tensor(np.ascontiguousarray(x), device=self.dev)
        rep = X.repeat_interleave(n_draws, dim=0).contiguous()
        o = self.forward(rep)
        z = torch.empty(rep.shape[0], 2, dtype=torch.float32, device=self.dev)
        check(lib.rbg_mdn_sample(o.data_ptr(), rep.shape[0], K, int(seed), z.data_ptr(), self._s()))
        c = torch.clamp(torch.round(torch.expm1(z)), min=0)
        return c.view(X.shape[0], n_draws, 2)

    def predict_params(self, x):
        """Mixture parameters at each query row (one forward pass): [Q][40]."""
        torch = self.torch
        X = torch.as_tensor(np.ascontiguousarray(x), device=self.dev)
        return self.forward(X.contiguous())


def wasserstein1(a: np.ndarray, b: np.ndarray) -> float:
    """W1 distance of two equal-size empirical samples (sorted differences)."""
    return float(np.mean(np.abs(np.sort(a) - np.sort(b))))


def ks_distance(a: np.ndarray, b: np.ndarray) -> float:
    grid = np.union1d(a, b)
    fa = np.searchsorted(np.sort(a), grid, side="right") / len(a)
    fb = np.searchsorted(np.sort(b), grid, side="right") / len(b)
    return float(np.max(np.abs(fa - fb)))

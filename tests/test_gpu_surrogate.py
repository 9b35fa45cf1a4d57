"""The learned surrogate's kernels: tensor-core GEMM against float64, the
network's loss and gradients against the CPU oracle, and a short training run
on engine-generated data."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def test_gemm_bf16_all_transposes(torch):
    from rebop_gb300._lib import check, lib

    rng = np.random.default_rng(0)
    for (M, N, K) in [(64, 64, 32), (100, 72, 40), (257, 130, 300), (40, 256, 4096)]:
        for ta in (0, 1):
            for tb in (0, 1):
                a = torch.tensor(rng.standard_normal((K, M) if ta else (M, K)), dtype=torch.bfloat16).cuda()
                b = torch.tensor(rng.standard_normal((N, K) if tb else (K, N)), dtype=torch.bfloat16).cuda()
                c = torch.empty(M, N, dtype=torch.float32, device="cuda")
                check(lib.rbg_mdn_gemm(a.data_ptr(), a.shape[1], ta, b.data_ptr(), b.shape[1], tb, c.data_ptr(), N,
                                       M, N, K, 0.0, torch.cuda.current_stream().cuda_stream))
                A = a.double().cpu().numpy()
                B = b.double().cpu().numpy()
                ref = (A.T if ta else A) @ (B.T if tb else B)
                err = np.abs(c.cpu().numpy() - ref).max() / (np.abs(ref).max() + 1e-30)
                assert err < 1e-5, (M, N, K, ta, tb, err)


@pytest.mark.parametrize("head", ["count", "mixture"])
def test_mdn_gradients_match_oracle(torch, head):
    from oracle import mdn_oracle
    from rebop_gb300 import surrogate as sg

    rng = np.random.default_rng(1)
    model = sg.MDN(seed=3, head=head)
    # network inputs: u (5), t, and the rate-equation log means (2)
    x = rng.uniform(-1, 1, size=(512, sg.N_IN)).astype(np.float32)
    x[:, 5] = rng.uniform(0, 1, 512)
    x[:, 6:] = rng.uniform(0, 8, (512, 2))
    # targets: counts (small ones and tail ones) and residuals
    n = np.where(rng.random((512, 2)) < 0.5, rng.integers(0, 31, (512, 2)), rng.integers(31, 5000, (512, 2)))
    y = np.concatenate([n, rng.normal(0.0, 0.3, size=(512, 2))], axis=1).astype(np.float32)
    model.x_mean = torch.tensor(x.mean(0)).cuda()
    model.x_std = torch.tensor(x.std(0) + 1e-6).cuda()
    loss, dW, db = model.loss_and_grad(torch.tensor(x).cuda(), torch.tensor(y).cuda())
    W = [w.double().cpu().numpy() for w in model.Wb]
    b = [v.double().cpu().numpy() for v in model.b]
    yo = y.astype(np.float64) if head == "count" else y[:, 2:].astype(np.float64)
    rl, rW, rb = mdn_oracle.forward_backward(W, b, x.astype(np.float64), yo, model.x_mean.double().cpu().numpy(),
                                             model.x_std.double().cpu().numpy(), head=head)
    assert abs(float(loss) - rl) <= 1e-3 * abs(rl) + 1e-4
    for i in range(len(W)):
        g, r = dW[i].double().cpu().numpy(), rW[i]
        assert np.linalg.norm(g - r) <= 2e-2 * np.linalg.norm(r) + 1e-7, ("dW", i)
        g, r = db[i].double().cpu().numpy(), rb[i]
        assert np.linalg.norm(g - r) <= 2e-2 * np.linalg.norm(r) + 1e-7, ("db", i)


def test_mdn_training_lowers_the_loss(torch):
    from rebop_gb300 import surrogate as sg

    x, y, _ = sg.generate(20000, seed=5, nb_steps=50)
    model = sg.MDN(seed=1)
    X, Y = sg.features(torch.tensor(x)), torch.tensor(y).cuda()
    model.x_mean, model.x_std = X.mean(0), X.std(0) + 1e-6
    before = float(model.loss_and_grad(X[:4096], Y[:4096])[0])
    model.fit(x, y, epochs=8, batch=1024, lr=3e-3)
    after = float(model.loss_and_grad(X[:4096], Y[:4096])[0])
    assert after < before - 0.5, (before, after)
    c = model.sample_counts(x[:16], 200).cpu().numpy()
    assert c.shape == (16, 200, 2) and (c >= 0).all()


def test_gemm_tcgen05_matches_float64(torch):
    # the tcgen05 / tensor-memory kernel against float64, all transposes
    from rebop_gb300._lib import check, lib

    rng = np.random.default_rng(2)
    err_flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    # (40, 256, 4096), (130, 72, 1100) and (256, 8, 4096) split K over the
    # grid; products of K-contiguous operands with rows 16-byte multiples apart
    # (ta = 0, tb = 1, K % 8 == 0) take the TMA-fed kernel -- (520, 200, 1000)
    # cycles its four-stage ring four times, (1000, 256, 8) reads one 8-wide
    # K slice, (4096, 112, 256) ends in a partial tile; beta != 0 checks the
    # accumulate epilogues
    shapes = [(128, 64, 64), (200, 100, 80), (4096, 256, 256), (40, 256, 4096), (256, 40, 256),
              (130, 72, 300), (64, 33, 27), (300, 96, 520), (130, 72, 1100), (256, 8, 4096),
              (520, 200, 1000), (1000, 256, 8), (4096, 112, 256)]
    for (M, N, K) in shapes:
        for ta in (0, 1):
            for tb in (0, 1):
                for beta in ((0.0, 0.5) if (ta, tb) in ((1, 0), (0, 1)) else (0.0,)):
                    a = torch.tensor(rng.standard_normal((K, M) if ta else (M, K)), dtype=torch.bfloat16).cuda()
                    b = torch.tensor(rng.standard_normal((N, K) if tb else (K, N)), dtype=torch.bfloat16).cuda()
                    c0 = rng.standard_normal((M, N))
                    c = torch.tensor(c0, dtype=torch.float32, device="cuda")
                    check(lib.rbg_mdn_gemm_tc05(a.data_ptr(), a.shape[1], ta, b.data_ptr(), b.shape[1], tb,
                                                c.data_ptr(), N, M, N, K, beta, err_flag.data_ptr(),
                                                torch.cuda.current_stream().cuda_stream))
                    torch.cuda.synchronize()
                    assert int(err_flag.item()) == 0
                    A = a.double().cpu().numpy()
                    B = b.double().cpu().numpy()
                    ref = (A.T if ta else A) @ (B.T if tb else B) + beta * c0.astype(np.float32)
                    err = np.abs(c.cpu().numpy() - ref).max() / (np.abs(ref).max() + 1e-30)
                    assert err < 1e-5, (M, N, K, ta, tb, beta, err)


@pytest.mark.parametrize("head", ["count", "mixture"])
def test_fused_inference_matches_layer_by_layer(torch, head):
    # rbg_mdn_infer (the whole MLP in one launch, activations in shared memory,
    # weights by TMA) against the layer-by-layer forward pass of the same
    # weights: one partial tile, several tiles, and more tiles than SMs
    from rebop_gb300 import surrogate as sg

    rng = np.random.default_rng(6)
    model = sg.MDN(seed=4, head=head)
    # non-trivial biases and input normalisation
    for b in model.b:
        b.copy_(torch.tensor(rng.normal(0, 0.1, b.shape[0]), dtype=torch.float32))
    model.x_mean = torch.tensor(rng.normal(0, 0.3, sg.N_IN), dtype=torch.float32).cuda()
    model.x_std = torch.tensor(rng.uniform(0.5, 2.0, sg.N_IN), dtype=torch.float32).cuda()
    for Q in (5, 1000, 70001):
        F = torch.tensor(rng.uniform(-2, 2, (Q, sg.N_IN)), dtype=torch.float32).cuda()
        fused = model.infer(F).cpu().numpy()
        ref = model.forward(F).cpu().numpy()
        model.check_errors()
        assert fused.shape == ref.shape == (Q, model.n_out)
        # the fused kernel's SiLU takes the fast reciprocal (the forward pass
        # an IEEE division): a hidden activation may round to the neighbouring
        # BF16 value (2^-8 relative), which moves an output by ~1e-3 of its
        # scale at most; nearly all outputs agree far closer
        scale = np.abs(ref).max()
        d = np.abs(fused - ref)
        assert d.max() <= 5e-3 * scale and d.mean() <= 1e-4 * scale, (Q, d.max(), d.mean(), scale)


def test_rate_equation_unrolled_kernel_equals_generic(torch):
    # The dimer's rate equations run on a kernel unrolled for 4 species and 5
    # reactions; the generic kernel on the same network with an idle fifth
    # species (no exponent, no change) must give the same bits.
    from rebop_gb300._lib import check, lib
    from rebop_gb300 import surrogate as sg

    rng = np.random.default_rng(9)
    Q = 3000
    rates = torch.tensor(np.asarray(sg.RATES0) * 10 ** rng.uniform(-1, 1, (Q, 5)), dtype=torch.float32).cuda()
    t = torch.tensor(rng.uniform(0.01, 1, Q), dtype=torch.float32).cuda()
    outs = []
    for S in (4, 5):
        E = np.zeros((5, S), np.int32)
        N = np.zeros((5, S), np.float32)
        E[:, :4], N[:, :4] = sg.EXPS, sg.DIFFS
        x0 = np.zeros(S, np.float32)
        x0[:4] = sg.X0
        Ed, Nd, x0d = (torch.tensor(v).cuda() for v in (E, N, x0))
        idx = torch.tensor([2, 3], dtype=torch.int32).cuda()
        out = torch.empty(Q, 2, dtype=torch.float32, device="cuda")
        check(lib.rbg_mdn_rre(rates.data_ptr(), t.data_ptr(), Q, S, 5, Ed.data_ptr(), Nd.data_ptr(), x0d.data_ptr(),
                              sg.RRE_STEPS, idx.data_ptr(), 2, out.data_ptr(),
                              torch.cuda.current_stream().cuda_stream))
        outs.append(out.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])


def _mix64(z):
    # SplitMix64's output function (Steele, Lea and Flood 2014), as the sampler hashes
    M = (1 << 64) - 1
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    return z ^ (z >> 31)


def test_count_sampler_follows_its_rule(torch):
    # rbg_mdn_count_sample: the prepared running sums equal the softmax's, every
    # below-tail draw is exactly #{k : cum_k <= u0} for its hashed uniform, and
    # tail draws are >= 31.
    from rebop_gb300._lib import check, lib
    from rebop_gb300 import surrogate as sg

    rng = np.random.default_rng(8)
    Q, per, KT = 24, 200, sg.KT
    HS = sg.NC + 3 * KT
    O = rng.normal(0, 2, (Q, 2 * HS)).astype(np.float32)
    O[:, sg.NC - 1] += 2.0  # a tail class that is drawn now and then
    o = torch.tensor(O).cuda()
    base = torch.tensor(rng.uniform(3, 5, (Q, 2)), dtype=torch.float32).cuda()
    out = torch.empty(Q * per, 2, dtype=torch.float32, device="cuda")
    work = torch.empty_like(o)
    seed = 12345
    check(lib.rbg_mdn_count_sample(o.data_ptr(), Q * per, KT, seed, out.data_ptr(), per, base.data_ptr(),
                                   work.data_ptr(), torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    W = work.cpu().numpy().reshape(Q, 2, HS)
    X = out.cpu().numpy()
    for q in range(Q):
        for sp in range(2):
            lg = O[q, sp * HS:sp * HS + sg.NC].astype(np.float64)
            pr = np.exp(lg - lg.max())
            np.testing.assert_allclose(W[q, sp, :sg.NC], np.cumsum(pr / pr.sum()), atol=2e-6)
    tails = 0
    for row in range(0, Q * per, 7):
        q = row // per
        for sp in range(2):
            h = _mix64(seed ^ _mix64(((row << 1 | sp) + 0x9E3779B97F4A7C15) & ((1 << 64) - 1)))
            u0 = np.float32((h >> 40) * 2.0 ** -24)
            c = min(int((W[q, sp, :sg.NC] <= u0).sum()), sg.NC - 1)
            if c < sg.NC - 1:
                assert X[row, sp] == c, (row, sp, X[row, sp], c)
            else:
                assert X[row, sp] >= sg.NC - 1
                tails += 1
    assert tails > 0


def test_rate_equation_kernel_matches_scipy(torch):
    # rbg_mdn_rre (float32 RK4, the surrogate's deterministic part) against an
    # adaptive float64 solution of the same rate equations
    from scipy.integrate import solve_ivp

    from rebop_gb300 import surrogate as sg

    rng = np.random.default_rng(4)
    x = np.concatenate([rng.uniform(-1, 1, (64, 5)), rng.uniform(0.01, 1, (64, 1))], axis=1).astype(np.float32)
    got = np.expm1(sg.rre_log_means(torch.tensor(x)).cpu().numpy().astype(np.float64))
    E, N = np.array(sg.EXPS, float), np.array(sg.DIFFS, float)
    for q in range(64):
        k = np.asarray(sg.RATES0) * 10.0 ** x[q, :5].astype(np.float64)

        def rhs(_, v):
            a = k.copy()
            for r in range(5):
                for s in range(4):
                    for j in range(int(E[r, s])):
                        a[r] *= max(v[s] - j, 0.0)
            return N.T @ a

        sol = solve_ivp(rhs, (0.0, float(x[q, 5])), np.array(sg.X0, float), method="LSODA", rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(got[q], sol.y[2:4, -1], rtol=2e-3, atol=1e-3)


def test_surrogate_accuracy_and_gain_over_ssa(torch):
    # The trained surrogate against the method without it, the plain GPU SSA,
    # on held-out (rates, t) points judged by fresh 1e4-trajectory SSA batches:
    # at the stated tolerance (W1 <= 1 % of the mean count) it answers queries
    # more than 50x faster than the SSA answers them with 1000 trajectories,
    # the majority of held-out points meet the tolerance for both species, the
    # gate answers the majority of random queries, and it answers exactly where
    # validation met the tolerance.
    import time

    from rebop_gb300 import surrogate as sg

    x, y, _ = sg.generate(1 << 22, seed=20260106)
    model = sg.MDN(seed=0)
    model.fit(x, y, epochs=20, batch=4096, lr=2e-3)
    sur = sg.Surrogate(model, tol=0.01)
    big = sur.validate(64, 10000, seed=8)
    w1 = big["w1"]
    assert np.median(w1[:, 0]) <= 0.01 and np.median(w1[:, 1]) <= 0.01, np.median(w1, axis=0)
    ok = (w1 <= 0.01).all(axis=1)
    assert ok.mean() >= 0.5, (ok.mean(), (big["w1_floor"] <= 0.01).all(axis=1).mean())
    rng = np.random.default_rng(9)
    qa = np.concatenate([rng.uniform(-1, 1, (100000, 5)), rng.integers(1, 101, (100000, 1)) / 100],
                        axis=1).astype(np.float32)
    assert sur.answer(qa).mean() >= 0.5
    # speed: 1000 draws per query against 1000 SSA trajectories per query
    rng = np.random.default_rng(3)
    q = np.concatenate([rng.uniform(-1, 1, (32768, 5)), rng.integers(1, 101, (32768, 1)) / 100],
                       axis=1).astype(np.float32)
    Q = torch.from_numpy(q).cuda()
    model.sample_counts(Q[:4096], 1000)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(0, 32768, 8192):
        model.sample_counts(Q[s:s + 8192], 1000)
    torch.cuda.synchronize()
    sur_qps = 32768 / (time.perf_counter() - t0)
    ssa_qps = 64 * 10 / (big["ssa_kernel_ms"] / 1e3)  # 1e4 trajectories per point: 10 queries of 1000
    assert sur_qps >= 50 * ssa_qps, (sur_qps, ssa_qps)
    # the gate answers exactly where validation met the tolerance
    assert np.array_equal(sur.answer(sur.points), ok)

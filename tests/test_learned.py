"""Learned smoother on the GPU: the network's forward pass and gradients
against the numpy oracle (same BF16 operand rounding; tolerance 2e-3
relative for FP32-accumulation order), training on harvested
(residual, error) pairs, and the solve with the learned post-smoothing step
(parity with the plain solver's solution, fallback to plain Vanka)."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def mlp():
    from to_merge_master_parmoon_gb300.learned import Mlp
    m = Mlp(device=0, seed=7, max_batch=512)
    yield m
    m.close()


def test_forward_and_gradients_match_oracle(mlp):
    import torch
    rng = np.random.default_rng(3)
    M = 96
    X = rng.standard_normal((M, mo.N_IN)).astype(np.float32)
    T = rng.standard_normal((M, mo.N_OUT)).astype(np.float32)
    P = mlp.params().astype(np.float64)
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    y_gpu = mlp.forward(Xd).cpu().numpy()
    y_ref, _ = mo.forward(P, X.astype(np.float64))
    assert rel(y_gpu, y_ref) < 2e-3
    loss, g = mlp.loss_grad(Xd, Td, want_grad=True)
    loss_ref, g_ref = mo.loss_grad(P, X.astype(np.float64), T.astype(np.float64))
    assert abs(loss - loss_ref) < 1e-4 * loss_ref
    blocks = [(mo.OFF_W1, mo.OFF_B1), (mo.OFF_B1, mo.OFF_W2), (mo.OFF_W2, mo.OFF_B2),
              (mo.OFF_B2, mo.OFF_W3), (mo.OFF_W3, mo.OFF_B3), (mo.OFF_B3, mo.N_PARAMS)]
    for a, b in blocks:
        assert rel(g[a:b], g_ref[a:b]) < 2e-3, (a, rel(g[a:b], g_ref[a:b]))


@pytest.mark.parametrize("M", [96, 300, 512])
def test_tcgen05_and_mma_sync_paths_agree(mlp, M):
    """The network's GEMMs on tcgen05 (TMEM accumulators, the default: the
    forward layers and the six backward products) and on mma.sync give the
    same outputs, loss and gradients (FP32 accumulation of the same BF16
    products in another order; tile edges at M not a multiple of 128 and
    batch sizes not a multiple of 64), and both match the oracle."""
    import torch
    rng = np.random.default_rng(M)
    X = rng.standard_normal((M, mo.N_IN)).astype(np.float32)
    T = rng.standard_normal((M, mo.N_OUT)).astype(np.float32)
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    P = mlp.params().astype(np.float64)
    y_ref, _ = mo.forward(P, X.astype(np.float64))
    out = {}
    for path in (True, False):
        mlp.set_tensor_path(path)
        y = mlp.forward(Xd).cpu().numpy()
        loss, g = mlp.loss_grad(Xd, Td, want_grad=True)
        out[path] = (y, loss, g)
        assert rel(y, y_ref) < 2e-3
    mlp.set_tensor_path(True)
    (y1, l1, g1), (y0, l0, g0) = out[True], out[False]
    assert rel(y1, y0) < 2e-3
    assert abs(l1 - l0) < 1e-4 * l0
    assert rel(g1, g0) < 2e-3


def test_adamw_step_matches_formula(mlp):
    import torch
    rng = np.random.default_rng(4)
    X = torch.from_numpy(rng.standard_normal((64, mo.N_IN)).astype(np.float32)).cuda()
    T = torch.from_numpy(rng.standard_normal((64, mo.N_OUT)).astype(np.float32)).cuda()
    from to_merge_master_parmoon_gb300.learned import Mlp
    m = Mlp(device=0, seed=11, max_batch=64)
    p0 = m.params().astype(np.float64)
    _, g = m.loss_grad(X, T, want_grad=True)
    m.adamw(lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=1e-2)
    p1 = m.params().astype(np.float64)
    g = g.astype(np.float64)
    mhat = g  # first step: bias-corrected moments equal g and g^2
    vhat = g * g
    bias = np.zeros(mo.N_PARAMS, bool)
    bias[mo.OFF_B1:mo.OFF_W2] = bias[mo.OFF_B2:mo.OFF_W3] = bias[mo.OFF_B3:] = True
    want = p0 - 1e-3 * (mhat / (np.sqrt(vhat) + 1e-8) + np.where(bias, 0.0, 1e-2 * p0))
    assert np.max(np.abs(p1 - want)) < 1e-6
    m.close()


@pytest.fixture(scope="module")
def trained(problems):
    from to_merge_master_parmoon_gb300.learned import Mlp, harvest_pairs, relative_loss, train
    Ps = [problems(3, nu, seed) for nu, seed in ((1e-2, 21), (3e-2, 22), (5e-3, 23))]
    X, T = harvest_pairs(Ps, n_cycles=6)
    m = Mlp(device=0, seed=5, max_batch=1024)
    before = relative_loss(m, X, T)
    hist = train(m, X, T, epochs=40, batch=512, lr=2e-3)
    after = relative_loss(m, X, T)
    yield m, X, T, before, after, hist
    m.close()


def test_harvest_and_training_reduce_loss(trained):
    m, X, T, before, after, hist = trained
    assert X.shape[1] == mo.N_IN and T.shape[1] == mo.N_OUT
    assert 0.9 * 3 * 512 * 6 <= X.shape[0] <= 3 * 512 * 6  # a few outlier rows may be dropped
    assert np.isfinite(hist).all()
    assert hist[-1] < 0.7 * hist[0], hist
    assert after < before, (before, after)


def test_learned_step_saves_an_iteration():
    """What the trained network gains: the benchmark's network (pairs from 8
    harvested 32^3 problems, 20 epochs, trained here on the GPU) on the 32^3
    Oseen problem of the benchmark's family (nu = 1e-2, seed 1) solved to
    1e-8 by FGMRES(20) with mixed-precision V(2,2) cycles: plain cell Vanka
    takes 10 iterations; with the learned post-smoothing step on the finest
    level the solve takes fewer, stays on (no fallback) and reaches the same
    solution to 1e-6."""
    from to_merge_master_parmoon_gb300 import OseenProblem, PmSolver
    from to_merge_master_parmoon_gb300.learned import standard_network
    net, info = standard_network(device=0)
    P = OseenProblem(n_levels=5, nu=1e-2, seed=1)
    b = P.rhs()
    nu3 = 3 * P.desc(4).n_udof
    bp = b.copy()
    bp[nu3::4] -= bp[nu3::4].mean()
    r0 = np.linalg.norm(bp)
    out = {}
    for name, m in (("plain", None), ("learned", net)):
        S = PmSolver(P.descs, precision="mixed", restart=20, maxit=80, res_norm_min=1e-8 * r0)
        if m is not None:
            S.attach_learned(m, omega=1.0, fallback_ratio=0.5)
        x, it = S.iterate(np.zeros_like(b), b)
        assert it["true_res"] <= 1.05e-8 * r0
        x[nu3::4] -= x[nu3::4].mean()
        out[name] = (it["iterations"], x, S.learned_status() if m is not None else None)
        S.close()
    net.close()
    print(f"learned step on 32^3, nu=1e-2: iterations {out['plain'][0]} -> "
          f"{out['learned'][0]} (training relative loss {info['relative_loss']:.2f})")
    assert out["learned"][2] == {"enabled": 1, "fallbacks": 0}
    assert out["learned"][0] < out["plain"][0]
    assert rel(out["learned"][1], out["plain"][1]) < 1e-6


def test_learned_solve_matches_plain_solution_and_falls_back(problems, trained):
    from to_merge_master_parmoon_gb300 import PmSolver
    m = trained[0]
    P = problems(3, 1e-2, 0)
    b = P.rhs()
    nu3 = 3 * P.desc(2).n_udof
    bp = b.copy()
    bp[nu3::4] -= bp[nu3::4].mean()
    tol = 1e-10 * np.linalg.norm(bp)
    plain = PmSolver(P.descs, precision="mixed", restart=20, maxit=80, res_norm_min=tol)
    x0, i0 = plain.iterate(np.zeros_like(b), b)
    S = PmSolver(P.descs, precision="mixed", restart=20, maxit=80, res_norm_min=tol)
    S.attach_learned(m, omega=1.0, fallback_ratio=0.5)
    x1, i1 = S.iterate(np.zeros_like(b), b)
    assert i1["true_res"] <= 1.05 * tol
    for v in (x0, x1):
        v[nu3::4] -= v[nu3::4].mean()
    assert rel(x1, x0) < 1e-6
    # a fallback ratio of 0 switches the learned step off after the first iteration
    S.attach_learned(m, omega=1.0, fallback_ratio=0.0)
    x2, i2 = S.iterate(np.zeros_like(b), b)
    st = S.learned_status()
    assert st["fallbacks"] >= 1 and st["enabled"] == 0
    assert i2["true_res"] <= 1.05 * tol
    S.attach_learned(None)
    S.close()
    plain.close()


def test_manufactured_harvest_matches_exact_solution_harvest(problems):
    """Pairs from a manufactured solution (b := K u*) equal the pairs of the
    exact-solution harvest when u* is that harvest's solution: the targets
    are the same errors, known without solving the system."""
    import torch
    from to_merge_master_parmoon_gb300 import PmSolver
    from to_merge_master_parmoon_gb300.learned import harvest_manufactured, harvest_pairs
    P = problems(3, 1e-2, 7)
    b = P.rhs()
    nu3 = 3 * P.desc(2).n_udof
    bp = b.copy()
    bp[nu3::4] -= bp[nu3::4].mean()
    S = PmSolver(P.descs, precision="fp64", restart=30, maxit=300,
                 res_norm_min=1e-11 * np.linalg.norm(bp))
    xs, _ = S.iterate(np.zeros_like(b), b)
    S.close()
    X1, T1 = harvest_pairs([P], n_cycles=3)
    X2, T2 = harvest_manufactured([P], n_cycles=3, solutions=[xs])
    assert X1.shape == X2.shape and T1.shape == T2.shape
    assert float(torch.linalg.norm(X1 - X2) / torch.linalg.norm(X1)) < 1e-3
    assert float(torch.linalg.norm(T1 - T2) / torch.linalg.norm(T1)) < 1e-3

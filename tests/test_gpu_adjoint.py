"""Adjoint gradients of <n_0(T)> with respect to the couplings of a
Bose-Hubbard chain (needs a GB300): against central finite differences on the
GPU and through the CPU oracle, and through torch.autograd."""
import numpy as np
import pytest

from oracle import models

pytestmark = pytest.mark.gpu


def _terms(L, N):
    states = models.basis(N, L)
    mats = []
    for b in range(L - 1):
        mats.append(models.create_matrix([models.lin_interaction(b, b + 1, 0, 0, False, -1.0),
                                          models.lin_interaction(b, b + 1, 0, 0, True, -1.0)], states))
    inter = []
    for i in range(L):
        inter += [models.four_point_a(i, i, i, i, 0, 0, 0, 0, 0.5), models.number_operator(i, -0.5)]
    mats.append(models.create_matrix(inter, states))
    return states, mats


def _sum(mats, theta):
    row = np.concatenate([m[0] for m in mats])
    col = np.concatenate([m[1] for m in mats])
    val = np.concatenate([th * m[2] for th, m in zip(theta, mats)])
    return row, col, val


@pytest.fixture(scope="module")
def problem(te_gpu):
    L, N = 5, 5
    states, mats = _terms(L, N)
    n = len(states)
    rng = np.random.default_rng(2)
    theta = np.concatenate([rng.uniform(0.8, 1.2, L - 1), [2.0]])
    v = np.zeros(n, dtype=np.complex128)
    v[models.index_of(states, [N] + [0] * (L - 1))] = 1.0
    O = models.create_matrix([models.number_operator(0, 1.0)], states)
    terms = [te_gpu.Matrix.from_coo(n, m) for m in mats]
    Om = te_gpu.Matrix.from_coo(n, O)
    adj = te_gpu.Adjoint(terms, Om, v, T=2.0, tol=1e-12, m=30, checkpoint_interval=0.5, nodes_per_interval=24)
    return dict(states=states, mats=mats, theta=theta, v=v, O=O, adj=adj, terms=terms, Om=Om)


def test_adjoint_matches_gpu_finite_differences(problem):
    adj, theta = problem["adj"], problem["theta"]
    loss, grad = adj.run(theta)
    assert abs(loss - adj.forward(theta)) < 1e-10
    h = 1e-5
    fd = np.zeros_like(theta)
    for k in range(len(theta)):
        e = np.zeros_like(theta)
        e[k] = h
        fd[k] = (adj.forward(theta + e) - adj.forward(theta - e)) / (2 * h)
    scale = np.max(np.abs(fd))
    assert np.max(np.abs(grad - fd)) < 1e-6 * scale, (grad, fd)


def test_adjoint_matches_oracle_finite_differences(problem, oracle_lib):
    adj, theta = problem["adj"], problem["theta"]
    _, grad = adj.run(theta)
    h = 1e-5
    for k in (0, len(theta) - 1):
        vals = []
        for sgn in (1, -1):
            th = theta.copy()
            th[k] += sgn * h
            r = oracle_lib.evolve(_sum(problem["mats"], th), problem["v"], 2.0, 2.0, [("sparse", problem["O"])],
                                  tol=1e-12, m=30)
            vals.append(r["samples"][0][-1])
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(grad[k] - fd) < 1e-6 * max(abs(fd), np.max(np.abs(grad))), (k, grad[k], fd)


def test_torch_autograd_binding(problem):
    torch = pytest.importorskip("torch")
    import timeevolver_gb300 as te
    adj, theta = problem["adj"], problem["theta"]
    f = te.expectation_function()
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    loss = f.apply(th, adj)
    loss.backward()
    ref_loss, ref_grad = adj.run(theta)
    assert abs(loss.item() - ref_loss) < 1e-14
    assert np.allclose(th.grad.numpy(), ref_grad, rtol=0, atol=1e-14)


def test_theta_refresh_is_stateless(problem):
    """H(theta) keeps one pattern and rescales its values on the device: the
    result for theta must not depend on the couplings used before."""
    adj, theta = problem["adj"], problem["theta"]
    l1, g1 = adj.run(theta)
    adj.run(theta * 1.3)
    adj.forward(theta[::-1].copy())
    l2, g2 = adj.run(theta)
    assert l1 == l2
    assert np.array_equal(g1, g2)


def test_forward_loss_matches_oracle(problem, oracle_lib):
    adj, theta = problem["adj"], problem["theta"]
    for th in (theta, 0.7 * theta[::-1].copy()):
        r = oracle_lib.evolve(_sum(problem["mats"], th), problem["v"], 2.0, 2.0, [("sparse", problem["O"])],
                              tol=1e-12, m=30)
        assert abs(adj.forward(th) - r["samples"][0][-1]) < 1e-9

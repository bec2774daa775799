"""GPU: multi-start hyperparameter search (rvgp_gp_fit_restarts) and the
many-fields sequence captured in a CUDA graph (main.ManyFieldsSolve).

* every restart of the batched launch follows the same trajectory as a
  single fit from its start (bitwise: the same kernel code per CTA or per
  thread-block cluster), its LML is the FP64 rvgp_gp_lml at its final
  parameters (1e-12), and the best one is the largest;
* replaying the captured graph gives the eager results (1e-12), and the
  batched posterior means equal per-field predict_fields at the best
  parameters (1e-10)."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def core():
    from rvgp_gb300 import _core
    _core.require_cuda()
    return _core


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def structured(seed, N, m):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((N, m)))
    Phi = Q * np.sqrt(N)
    lam = np.sort(rng.uniform(0.0, 3.0, m))
    coef = rng.standard_normal(m) / (1.0 + lam) ** 2
    return Phi, Phi @ coef + 0.05 * rng.standard_normal(N), lam


@pytest.mark.parametrize("m,N,R,force_cluster", [(60, 900, 5, False), (60, 900, 3, True), (300, 5000, 3, False),
                                                      (600, 9000, 2, False)])
def test_restarts_equal_single_fits(core, m, N, R, force_cluster):
    if m > core.gp_fit_mixed_max_m():
        pytest.skip("m beyond the mixed fit on this device")
    Phi, y, lam = structured(4, N, m)
    C, b, yy = core.gp_prepare(cu(Phi), cu(y))
    rng = np.random.default_rng(1)
    th0 = np.tile([1.5, 5.0, 1.0, 1.0], (R, 1))
    th0[:, 1] = np.exp(rng.uniform(np.log(0.5), np.log(50.0), R))
    lower = cu([0.0, 0.0, 0.0, 1e-6])
    mask = torch.tensor([1, 1, 1, 1], dtype=torch.int32, device="cuda")
    old = os.environ.get("RVGP_GP_FIT_CLUSTER")
    os.environ["RVGP_GP_FIT_CLUSTER"] = "1" if force_cluster else "0"
    try:
        out = core.gp_fit_restarts(C, b, yy, N, cu(lam), 3.0 * N, cu(th0), lower, mask, 80, history=True)
        singles = [core.gp_fit_adam_mixed(C, b, yy, N, cu(lam), 3.0 * N, cu(th0[r]), [0.0, 0.0, 0.0, 1e-6],
                                          [1, 1, 1, 1], 80, history=True) for r in range(R)]
    finally:
        if old is None:
            del os.environ["RVGP_GP_FIT_CLUSTER"]
        else:
            os.environ["RVGP_GP_FIT_CLUSTER"] = old
    th = out["theta"].cpu().numpy()
    lml = out["lml"].cpu().numpy()
    for r in range(R):
        assert singles[r][4]
        np.testing.assert_array_equal(th[r], singles[r][0].cpu().numpy())
        np.testing.assert_array_equal(out["hist"][r].cpu().numpy(), singles[r][2].cpu().numpy())
        ref, _ = core.gp_lml(C, b, yy, N, cu(lam), 3.0 * N, cu(th[r]))
        np.testing.assert_allclose(lml[r], ref.cpu().numpy()[0], rtol=1e-12)
    best = int(out["best"].cpu().numpy()[0])
    assert best == int(np.argmax(lml))
    np.testing.assert_array_equal(out["theta_best"].cpu().numpy(), th[best])


def test_many_fields_graph_replay_equals_eager():
    import rvgp_gb300 as RVGP
    from rvgp_gb300.main import ManyFieldsSolve
    from rvgp_gb300.workloads import make_points
    n, m, B = 1500, 40, 24
    X = make_points("half_ellipsoid", n, seed=2)
    d = RVGP.create_data_object(X, n_neighbors=12, n_eigenpairs=m, verbose=False)
    rng = np.random.default_rng(3)
    fields = torch.as_tensor(rng.standard_normal((B, n, 3)), device="cuda")
    d.vectors = fields[0]
    train = np.sort(rng.choice(n, 64, replace=False))
    test = np.setdiff1d(np.arange(n), train)
    gp = RVGP.fit(d, train_ind=train, epochs=0, verbose=False)
    solve = ManyFieldsSolve(gp, fields, test, gp.restart_starts(6, seed=4), epochs=60)
    solve.enqueue()
    torch.cuda.synchronize()
    eager_mean, eager_lml = solve.mean.clone(), solve.lml.clone()
    eager_theta = solve.fit["theta_best"].clone()
    solve.capture()
    solve.mean.zero_()
    solve.lml.zero_()
    solve.replay()
    torch.cuda.synchronize()
    assert torch.equal(solve.fit["theta_best"], eager_theta)
    np.testing.assert_allclose(solve.mean.cpu().numpy(), eager_mean.cpu().numpy(), rtol=0,
                               atol=1e-12 * float(eager_mean.abs().max()))
    np.testing.assert_allclose(solve.lml.cpu().numpy(), eager_lml.cpu().numpy(), rtol=1e-12)
    # the best parameters are the largest FP64 likelihood, and the batched
    # posterior equals predict_fields with them
    lml = solve.fit["lml"].cpu().numpy()
    assert int(solve.fit["best"].cpu().numpy()[0]) == int(np.argmax(lml))
    for p, v in zip(gp._slots(), eager_theta.cpu().numpy()):
        if p is not None:
            p.assign(float(v))
    ref, ref_lml = gp.predict_fields(fields, test)
    got = solve.means()
    np.testing.assert_allclose(got.cpu().numpy(), ref.cpu().numpy(), rtol=0,
                               atol=1e-10 * float(ref.abs().max()))
    np.testing.assert_allclose(solve.lml.cpu().numpy(), ref_lml.cpu().numpy(), rtol=1e-10)

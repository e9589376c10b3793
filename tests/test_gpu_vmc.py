"""End-to-end VMC on the GPU: expect / expect_and_grad against the oracle on
the same sample set, the gradient against an exact full-sum gradient, and the
1D transverse-field Ising chain (N=16, h=J=1) converging to the Lanczos
ground-state energy."""
import numpy as np
import pytest
import torch

from gpu_common import oracle_heisenberg, oracle_params
from oracle import exact as oex
from oracle import operator as oop
from oracle import rbm as orbm
from oracle import stats as ost

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nk():
    import netket_gb300
    netket_gb300._native.require_cuda()
    return netket_gb300


def test_expect_and_grad_matches_oracle(nk):
    L = 4
    g = nk.graph.Square(L)
    hi = nk.hilbert.Spin(0.5, N=16, total_sz=0)
    H = nk.operator.Heisenberg(hi, g)
    vs = nk.vqs.MCState(nk.sampler.MetropolisExchange(hi, graph=g, n_chains=64),
                        nk.models.RBM(alpha=2), n_samples=2048, seed=2, precision="fp64")
    st, grad = vs.expect_and_grad(H)
    s = vs.samples.reshape(-1, 16).cpu().numpy()
    p = oracle_params(vs.flat_parameters, 16, vs.M)
    e = orbm.local_energies(p, s, oracle_heisenberg(g).get_conn_padded)
    ref_stats = ost.statistics(e.reshape(64, -1))
    np.testing.assert_allclose(st.as_array(), ref_stats.as_array(), rtol=1e-10, equal_nan=True)
    _, ref_grad = orbm.forces_and_grad(p, s, e)
    got = vs.model.flatten(grad).cpu().numpy()
    np.testing.assert_allclose(got, ref_grad, rtol=1e-9, atol=1e-11 * np.abs(ref_grad).max())
    F_stats, F = vs.expect_and_forces(H)
    np.testing.assert_array_equal(2 * vs.model.flatten(F).cpu().numpy(), got)


def test_gradient_matches_full_sum(nk):
    """Monte Carlo gradient within 5 sigma-ish of the exact gradient (N=10)."""
    N = 10
    g = nk.graph.Chain(N)
    hi = nk.hilbert.Spin(0.5, N)
    H = nk.operator.Ising(hi, g, h=0.9)
    model = nk.models.RBM(alpha=1, kernel_init_std=0.2, hidden_bias_init_std=0.2,
                          visible_bias_init_std=0.2)
    vs = nk.vqs.MCState(nk.sampler.MetropolisLocal(hi, n_chains=512), model, n_samples=512 * 256,
                        n_discard_per_chain=64, seed=3, precision="fp64")
    st, grad = vs.expect_and_grad(H)
    p = oracle_params(vs.flat_parameters, N, vs.M)
    E, G = oex.full_sum_energy_and_grad(
        p, lambda s: oop.ising_get_conn_padded(s, np.array(g.edges()), 0.9, 1.0), N)
    assert abs(st.mean - E) < 5 * st.error_of_mean + 1e-3
    got = vs.model.flatten(grad).cpu().numpy()
    assert np.linalg.norm(got - G) < 0.05 * np.linalg.norm(G) + 5e-3


@pytest.mark.slow
def test_tfim_chain16_vmc_sr_converges(nk):
    """Configuration of the 1D TFIM benchmark: N=16, J=1, h=1, RBM alpha=1 FP64,
    MetropolisLocal 16 chains, 1008 samples, 32 discarded sweeps, SR
    diag_shift=0.01, sgd lr=0.01.  After 300 steps the energy is within 1% of
    the exact ground state (NetKet's RBM reaches the same band)."""
    N = 16
    g = nk.graph.Chain(N)
    hi = nk.hilbert.Spin(0.5, N)
    H = nk.operator.Ising(hi, g, h=1.0, J=1.0)
    E0 = oex.lanczos_ed(lambda s: oop.ising_get_conn_padded(s, np.array(g.edges()), 1.0, 1.0), N)[0]
    assert abs(E0 - oex.tfim_ground_energy(N, 1.0, 1.0)) < 1e-8
    vs = nk.vqs.MCState(nk.sampler.MetropolisLocal(hi, n_chains=16), nk.models.RBM(alpha=1),
                        n_samples=1008, n_discard_per_chain=32, seed=0, precision="fp64")
    drv = nk.driver.VMC(H, nk.optimizer.Sgd(0.01), variational_state=vs,
                        preconditioner=nk.optimizer.SR(qgt="dense", diag_shift=0.01))
    log = nk.logging.RuntimeLog()
    drv.run(300, out=log)
    tail = log["Energy"]["Mean"][-50:]
    assert abs(tail.mean() - E0) / abs(E0) < 1e-2
    # the state's own estimate with more samples
    st = vs.expect(H)
    assert abs(st.mean - E0) / abs(E0) < 1e-2


def _j1j2(nk, L, alpha, n_chains, n_samples, seed, precision):
    """L x L J1-J2 (J2/J1 = 0.5, Marshall sign on J1, Sz = 0), RBM alpha, Exchange
    sampler on the nn + nnn clusters, minSR with diag_shift 1e-4, SGD lr 0.01."""
    g = nk.graph.Square(L, max_neighbor_order=2)
    hi = nk.hilbert.Spin(0.5, N=L * L, total_sz=0)
    H = nk.operator.Heisenberg(hi, g, J=[1.0, 0.5], sign_rule=[True, False])
    vs = nk.vqs.MCState(nk.sampler.MetropolisExchange(hi, graph=g, d_max=1, n_chains=n_chains),
                        nk.models.RBM(alpha=alpha), n_samples=n_samples, n_discard_per_chain=5,
                        seed=seed, precision=precision)
    drv = nk.driver.VMC_SR(H, nk.optimizer.Sgd(0.01), diag_shift=1e-4, variational_state=vs,
                           use_ntk=True)
    return H, vs, drv


def _pin_samples(vs):
    """Make ``vs`` take its samples from ``box["x"]`` instead of its sampler."""
    box = {}
    vs.reset = lambda: None

    def sample(**kw):
        vs._samples = box["x"]
        return vs._samples
    vs.sample = sample
    return box


def test_vmc_sr_minsr_step_mixed_matches_fp64(nk):
    """One minSR step at the benchmark's shape (10x10 J1-J2, alpha 4, M = 400) with
    4,096 samples: the mixed path (FP32 sampler / local-energy kernels, tensor-core
    Gram of t - s0 on a 2^-19 grid, FP32 factor refined to an FP64 residual) on
    the FP64 path's samples.  Bounds: energy 1e-7 relative, update 1.2e-4
    relative (measured on a GB300: 1.2e-8 and 1.1e-5; with the BF16 hi + lo Gram,
    gram_mode 2, 2.9e-5: the Gram matrix of the rounded Jacobian differs from
    the FP64 one by ~1e-6 relative, and minSR amplifies it by the conditioning of
    T at diag_shift 1e-4)."""
    _, vs64, drv64 = _j1j2(nk, 10, 4, 1024, 4096, 1, "fp64")
    H, vsm, drvm = _j1j2(nk, 10, 4, 1024, 4096, 1, "mixed")
    box = _pin_samples(vsm)
    drv64.advance(2)
    vsm.flat_parameters = vs64.flat_parameters.clone()
    s64, d64 = drv64.compute_loss_and_update()
    box["x"] = vs64.samples.clone()
    sm, dm = drvm.compute_loss_and_update()
    assert drvm.info["status"] == 0
    e_err = abs(sm.mean - s64.mean) / abs(s64.mean)
    d64, dm = d64.cpu().numpy(), dm.cpu().numpy()
    u_err = np.linalg.norm(dm - d64) / np.linalg.norm(d64)
    print(f"mixed vs fp64 at n=4096: energy {e_err:.3e}, update {u_err:.3e}")
    assert e_err < 1e-7, e_err
    assert u_err < 1.2e-4, u_err


def _heisenberg16(nk, precision, seed):
    """The large configuration's model at 4,096 samples: 16x16 Heisenberg (J = 1,
    Marshall sign, Sz = 0), RBM alpha 8 (M = 2048), Exchange sampler on the nn
    clusters, minSR with diag_shift 1e-4, SGD lr 0.005."""
    g = nk.graph.Square(16)
    hi = nk.hilbert.Spin(0.5, N=256, total_sz=0)
    H = nk.operator.Heisenberg(hi, g, J=1.0, sign_rule=True)
    vs = nk.vqs.MCState(nk.sampler.MetropolisExchange(hi, graph=g, n_chains=1024),
                        nk.models.RBM(alpha=8), n_samples=4096, n_discard_per_chain=5,
                        seed=seed, precision=precision)
    drv = nk.driver.VMC_SR(H, nk.optimizer.Sgd(0.005), diag_shift=1e-4, variational_state=vs,
                           use_ntk=True)
    return H, vs, drv


def test_minsr_step_mixed_matches_fp64_at_alpha8(nk):
    """One minSR step of the large configuration's model (16x16, alpha 8, M =
    2048) at 4,096 samples: the mixed path -- the Exchange kernel that reads W
    through L2, x W and O^T v on tcgen05, the mode-4 tensor-core Gram (M > 512),
    the FP32 factor refined to an FP64 residual -- on the FP64 path's samples,
    after two FP64 steps.  Bounds: energy 1e-7 relative, update 1e-4 relative
    (measured on a GB300: 3.1e-8 and 1.8e-5)."""
    _, vs64, drv64 = _heisenberg16(nk, "fp64", 2)
    _, vsm, drvm = _heisenberg16(nk, "mixed", 2)
    box = _pin_samples(vsm)
    drv64.advance(2)
    vsm.flat_parameters = vs64.flat_parameters.clone()
    s64, d64 = drv64.compute_loss_and_update()
    box["x"] = vs64.samples.clone()
    sm, dm = drvm.compute_loss_and_update()
    assert drvm.info["status"] == 0
    e_err = abs(sm.mean - s64.mean) / abs(s64.mean)
    d64, dm = d64.cpu().numpy(), dm.cpu().numpy()
    u_err = np.linalg.norm(dm - d64) / np.linalg.norm(d64)
    print(f"mixed vs fp64 at 16x16 alpha 8, n=4096: energy {e_err:.3e}, update {u_err:.3e}")
    assert e_err < 1e-7, e_err
    assert u_err < 1e-4, u_err


def test_mixed_trajectory_tracks_fp64(nk):
    """Matched energy error: 50 minSR steps of a 6x6 J1-J2 model (alpha 2, 1,024
    samples) from the same initial parameters.  The mixed run takes the FP64 run's
    samples at every step (its own parameters, its own FP32 kernels and refined
    solve), so the two energies differ only by arithmetic; they stay within 1e-4
    relative of each other at every step while the energy falls (measured on a
    GB300: 2.2e-5 at worst)."""
    _, vs64, drv64 = _j1j2(nk, 6, 2, 256, 1024, 3, "fp64")
    _, vsm, drvm = _j1j2(nk, 6, 2, 256, 1024, 3, "mixed")
    box = _pin_samples(vsm)
    vsm.flat_parameters = vs64.flat_parameters.clone()
    worst, energies = 0.0, []
    for step in range(50):
        s64, d64 = drv64.compute_loss_and_update()
        box["x"] = vs64.samples.clone()
        drv64.update_parameters(d64)
        drv64.step_count += 1
        sm, dm = drvm.compute_loss_and_update()
        drvm.update_parameters(dm)
        drvm.step_count += 1
        worst = max(worst, abs(sm.mean - s64.mean) / abs(s64.mean))
        energies.append(s64.mean)
    print(f"mixed vs fp64 over 50 steps: worst energy deviation {worst:.3e}")
    assert energies[-1] < energies[0]
    assert worst < 1e-4, worst


def test_vmc_sr_onthefly_tracks_dense_sr(nk):
    """VMC + SR on the 1D TFIM (N = 16): the QGTOnTheFly + CG preconditioner with a
    tight tolerance gives the same trajectory as the dense QGT for 10 steps."""
    N = 16
    g = nk.graph.Chain(N)
    hi = nk.hilbert.Spin(0.5, N)
    H = nk.operator.Ising(hi, g, h=1.0, J=1.0)
    params = []
    for qgt in ("dense", "onthefly"):
        vs = nk.vqs.MCState(nk.sampler.MetropolisLocal(hi, n_chains=16), nk.models.RBM(alpha=1),
                            n_samples=1008, n_discard_per_chain=32, seed=0, precision="fp64")
        sr = nk.optimizer.SR(diag_shift=0.01, qgt=qgt, tol=1e-12)
        drv = nk.driver.VMC(H, nk.optimizer.Sgd(0.01), variational_state=vs, preconditioner=sr)
        drv.run(10)
        params.append(vs.flat_parameters.cpu().numpy())
    np.testing.assert_allclose(params[1], params[0], rtol=1e-7, atol=1e-9)


def test_checkpoint_resume_continues_chains_exactly(nk):
    """to_bytes / from_bytes (flax.serialization as NetKet uses it): a state
    restored into a fresh MCState continues parameters, chains and random stream
    bit for bit."""
    N = 12
    g = nk.graph.Chain(N)
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    H = nk.operator.Heisenberg(hi, g)

    def make():
        vs = nk.vqs.MCState(nk.sampler.MetropolisExchange(hi, graph=g, n_chains=32),
                            nk.models.RBM(alpha=1), n_samples=256, seed=3, precision="fp64")
        drv = nk.driver.VMC(H, nk.optimizer.Sgd(0.02), variational_state=vs,
                            preconditioner=nk.optimizer.SR(qgt="dense", diag_shift=0.01))
        return vs, drv
    vs, drv = make()
    drv.run(3)
    blob = nk.serialization.to_bytes(vs)
    drv.run(2)
    ref = vs.flat_parameters.cpu().numpy().copy()
    ref_samples = vs.sample().cpu().numpy()
    vs2, drv2 = make()
    nk.serialization.from_bytes(vs2, blob)
    drv2.run(2)
    np.testing.assert_array_equal(vs2.flat_parameters.cpu().numpy(), ref)
    np.testing.assert_array_equal(vs2.sample().cpu().numpy(), ref_samples)


def test_expect_to_precision_reaches_tolerance(nk):
    """expect_to_precision (netket/_src/vqs/expect_to_precision.py): sampling rounds
    continue until the error of the mean meets atol; the estimate is within 5
    sigma of the exact expectation value (full sum)."""
    N = 8
    g = nk.graph.Chain(N)
    hi = nk.hilbert.Spin(0.5, N)
    H = nk.operator.Ising(hi, g, h=1.0, J=1.0)
    model = nk.models.RBM(alpha=1, kernel_init_std=0.3, hidden_bias_init_std=0.3,
                          visible_bias_init_std=0.3)
    vs = nk.vqs.MCState(nk.sampler.MetropolisLocal(hi, n_chains=64), model, n_samples=512,
                        seed=2, precision="fp64")
    acc = vs.expect_to_precision(H, atol=2e-3)
    st = acc.get_stats()
    assert st.error_of_mean <= 2e-3 and vs.last_precision_rounds >= 1
    assert acc.n_samples == 512 * (vs.last_precision_rounds + 1)
    # exact expectation from the full sum over the 256 configurations
    allx = torch.as_tensor(hi.all_states(), device="cuda")
    lp = vs.log_value(allx)
    w = torch.exp(2 * (lp - lp.max()))
    w = w / w.sum()
    e = nk.kernels.local_energies_fused(H, vs.flat_parameters, allx, N, vs.M)
    exact = float((w * e).sum())
    assert abs(st.mean - exact) < 5 * st.error_of_mean
    with pytest.raises(ValueError):
        vs.expect_to_precision(H)
    # a dict of operators: one accumulator each, returned under the same keys
    Z = nk.operator.LocalOperator(hi, [np.array([[1.0, 0.0], [0.0, -1.0]])], [[0]])
    res = vs.expect_to_precision({"H": H, "Z": Z}, rtol=0.05, max_iter=50)
    assert set(res) == {"H", "Z"}
    assert res["H"].get_stats().error_of_mean <= 0.05 * abs(res["H"].mean)


def test_vmc_sr_linear_solver_choices(nk):
    """VMC_SR(linear_solver=cholesky / pinv_smooth) and the accepted NetKet
    arguments (MCState chunk_size, chunk_size_bwd, on_the_fly): the plain
    Cholesky step equals the default step bit for bit on an SPD system, the
    pinv_smooth step agrees to 1e-8."""
    N = 8
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    H = nk.operator.Heisenberg(hi, nk.graph.Chain(N))

    def step(**kw):
        vs = nk.vqs.MCState(nk.sampler.MetropolisExchange(hi, graph=nk.graph.Chain(N),
                                                          n_chains=64),
                            nk.models.RBM(alpha=1), n_samples=256, seed=4, precision="fp64",
                            chunk_size=32)
        drv = nk.driver.VMC_SR(H, nk.optimizer.Sgd(0.02), diag_shift=1e-2, variational_state=vs,
                               use_ntk=True, chunk_size_bwd=16, on_the_fly=True, **kw)
        drv.advance(1)
        return vs.flat_parameters.clone()

    a = step()
    b = step(linear_solver=nk.optimizer.solver.cholesky)
    c = step(linear_solver=nk.optimizer.solver.pinv_smooth)
    assert torch.equal(a, b)
    torch.testing.assert_close(c, a, rtol=1e-8, atol=1e-10)

"""Batched VMC over independent TFIM chains of uneven size: every instance's
parameters after eager and graph-replayed batched steps are bit-identical to
running that instance alone through MCState + VMC_SR with the same seeds."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nk():
    import netket_gb300
    netket_gb300._native.require_cuda()
    return netket_gb300


def _single(nk, N, h, seed, steps, B, L, nd, shift, lr):
    hi = nk.hilbert.Spin(0.5, N)
    H = nk.operator.Ising(hi, nk.graph.Chain(N), h=h)
    vs = nk.vqs.MCState(nk.sampler.MetropolisLocal(hi, n_chains=B),
                        nk.models.RBM(alpha=2, param_dtype=torch.float32), n_samples=B * L,
                        n_discard_per_chain=nd, seed=seed, sampler_seed=seed + 1,
                        precision="mixed")
    drv = nk.driver.VMC_SR(H, nk.optimizer.Sgd(lr), diag_shift=shift, variational_state=vs,
                           use_ntk=True, gram_mode=1, solve="refined")
    energies = []
    for _ in range(steps):
        energies.append(drv.advance(1).mean)
    return vs.flat_parameters.clone(), energies


def test_batched_equals_single(nk, tmp_path, monkeypatch):
    monkeypatch.setenv("VMCK_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    inst = [(8, 0.7), (12, 1.1), (16, 0.9), (24, 1.3)]
    B, L, nd, shift, lr = 64, 4, 5, 1e-4, 0.01
    bt = nk.batched.BatchedTFIM(inst, n_chains=B, chain_length=L, n_discard=nd,
                                diag_shift=shift, lr=lr, seed=10)
    e_b = []
    for _ in range(2):
        st, status = bt.step()
        assert np.all(status == 0)
        e_b.append([s.mean for s in st])
    bt.capture()  # runs one eager step, then captures
    e_b.append(list(bt.stats[:, 0].cpu().numpy()))
    for _ in range(2):
        st, status = bt.step()
        assert np.all(status == 0)
        e_b.append([s.mean for s in st])
    steps = bt.step_count
    assert steps == 5
    for i, (N, h) in enumerate(inst):
        p, e = _single(nk, N, h, 10 + i, steps, B, L, nd, shift, lr)
        assert torch.equal(p, bt.instance_parameters(i)), f"instance {i} differs"
        np.testing.assert_array_equal(np.array(e), np.array([row[i] for row in e_b]))


def test_batched_equals_single_at_workload_size(nk, tmp_path, monkeypatch):
    """Three instances of the 64-instance workload's distribution, at its sizes
    (1024 chains x 4 samples, the largest N = 144 among them), stepped by the
    batched runner (two eager steps and one captured-graph step) equal their
    single-instance runs bit for bit."""
    monkeypatch.setenv("VMCK_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    full = nk.batched.tfim_instances(64, seed=0)
    big = max(full, key=lambda t: t[0])
    small = min(full, key=lambda t: t[0])
    inst = [big, full[1], small]
    B, L, nd, shift, lr = 1024, 4, 5, 1e-4, 0.01
    bt = nk.batched.BatchedTFIM(inst, n_chains=B, chain_length=L, n_discard=nd,
                                diag_shift=shift, lr=lr, seed=20)
    for _ in range(2):
        _, status = bt.step()
        assert np.all(status == 0)
    bt.capture()
    _, status = bt.step()
    assert np.all(status == 0)
    for i, (N, h) in enumerate(inst):
        p, _ = _single(nk, N, h, 20 + i, bt.step_count, B, L, nd, shift, lr)
        assert torch.equal(p, bt.instance_parameters(i)), f"instance {i} (N={N}) differs"

"""Metropolis sampling on the GPU.  As in NetKet (test/sampler/test_sampler.py:
400-458) parity is distributional: the histogram of samples on a small system
must follow |psi|^2 (chi-squared, Fisher-combined p-value > 0.01).  Also:
determinism, Sz conservation, acceptance bookkeeping, log_prob consistency."""
import numpy as np
import pytest
import torch
from scipy import stats as sps

from gpu_common import oracle_params
from oracle import hilbert as oh
from oracle import rbm as orbm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nk():
    import netket_gb300
    netket_gb300._native.require_cuda()
    return netket_gb300


def _chi2_pvalues(nk, make_sampler, model, flat, N, total_sz, dtype, reps=6, independent=True):
    """Fisher-combined chi-squared p-value of the sample histogram against |psi|^2.

    independent=True: one sample per chain per repetition, 30 sweeps apart, with
    many chains -- the samples inside a repetition are independent, so the test
    stays valid for strongly peaked distributions.  independent=False: NetKet's
    form (consecutive samples of 64 chains, n_samples = 40 * n_states), valid
    for near-uniform distributions only."""
    states = oh.all_states(N, total_sz)
    p = oracle_params(flat, N, model.n_hidden(N))
    lp = orbm.logpsi(p, states)
    prob = np.exp(2 * (lp - lp.max()))
    prob /= prob.sum()
    w = 2 ** np.arange(N - 1, -1, -1)
    code = {int(c): i for i, c in enumerate(oh.states_to_local_indices(states).astype(np.int64) @ w)}
    n_samples = max(40 * len(states), 100)
    n_chains = n_samples if independent else 64
    sampler = make_sampler(n_chains)
    chain_length = 1 if independent else int(np.ceil(n_samples / n_chains))
    n_discard = 30 if independent else 0
    pvals = []
    params = flat.to(dtype)
    state = sampler.init_state(model, params, seed=123)
    samples, state = sampler.sample(model, params, state=state, chain_length=1, n_discard=50)
    for _ in range(reps):
        samples, state = sampler.sample(model, params, state=state, chain_length=chain_length,
                                        n_discard=n_discard)
        s = samples.reshape(-1, N).cpu().numpy()
        idx = np.array([code[int(c)] for c in oh.states_to_local_indices(s).astype(np.int64) @ w])
        hist = np.bincount(idx, minlength=len(states))
        pvals.append(sps.chisquare(hist, prob * len(idx)).pvalue)
    return sps.combine_pvalues(pvals, method="fisher").pvalue


def _model(nk, std):
    return nk.models.RBM(alpha=1, kernel_init_std=std, hidden_bias_init_std=std,
                         visible_bias_init_std=std)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("std,independent", [(0.1, False), (0.5, True)])
def test_local_rule_distribution(nk, dtype, std, independent):
    N = 6
    model = _model(nk, std)
    flat = model.init_flat(7, N)
    hi = nk.hilbert.Spin(0.5, N)
    make = lambda nc: nk.sampler.MetropolisLocal(hi, n_chains=nc)
    assert _chi2_pvalues(nk, make, model, flat, N, None, dtype, independent=independent) > 0.01


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("std,independent", [(0.1, False), (0.5, True)])
def test_exchange_rule_distribution(nk, dtype, std, independent):
    N = 8
    model = _model(nk, std)
    flat = model.init_flat(8, N)
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    g = nk.graph.Chain(N, max_neighbor_order=2)
    make = lambda nc: nk.sampler.MetropolisExchange(hi, graph=g, d_max=1, n_chains=nc)
    assert len(make(1).rule.clusters) == 16
    assert _chi2_pvalues(nk, make, model, flat, N, 0, dtype, independent=independent) > 0.01


@pytest.mark.parametrize("alpha,std", [(20, 0.12), (40, 0.09), (60, 0.07)])
def test_exchange_smem_kernel_wide_hidden_layer_distribution(nk, alpha, std):
    """The shared-memory Exchange kernel keeps M / 32 hidden units per lane in
    registers and is instantiated for up to 4, 8, 13 and 16 of them.  M = 160,
    320 and 480 (N = 8, Sz = 0, FP32) reach the 8-, 13- and 16-unit forms; the
    13-unit form is the one the 10x10 alpha = 4 workload (M = 400) runs.  The
    sample histogram must follow |psi|^2."""
    N = 8
    model = nk.models.RBM(alpha=alpha, kernel_init_std=std, hidden_bias_init_std=std,
                          visible_bias_init_std=std)
    flat = model.init_flat(21, N)
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    g = nk.graph.Chain(N, max_neighbor_order=2)
    make = lambda nc: nk.sampler.MetropolisExchange(hi, graph=g, d_max=1, n_chains=nc)
    assert _chi2_pvalues(nk, make, model, flat, N, 0, torch.float32, independent=True) > 0.01


@pytest.mark.parametrize("L,alpha", [(10, 4), (10, 1), (10, 2), (6, 14), (10, 8), (16, 8),
                                     (6, 40)])
def test_exchange_smem_kernel_matches_generic_kernel(nk, monkeypatch, L, alpha):
    """At the benchmark's shape (10x10, nn + nnn clusters, FP32; M = 100, 200 and
    400: the 4-, 8- and 13-unit forms) and on 6x6 with M = 504 (the 16-unit form;
    at N = 100 its weights would not fit in shared memory) the shared-memory
    Exchange kernel draws the same random numbers and evaluates the same
    floating-point expressions as the generic warp-per-chain kernel: samples,
    log-probabilities and acceptance counters are identical.  The same holds for
    the kernel that reads wider weights through L2: 10x10 alpha 8 (M = 800, 32
    units per lane), 16x16 alpha 8 (M = 2048, the large configuration's model;
    64 units) and 6x6 alpha 40 (M = 1440, a partly filled 64-unit form)."""
    N = L * L
    model = nk.models.RBM(alpha=alpha)
    flat = model.init_flat(4, N).float()
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    g = nk.graph.Square(L, max_neighbor_order=2)
    out = []
    for generic in ("0", "1"):
        monkeypatch.setenv("VMCK_EXCHANGE_GENERIC", generic)
        sampler = nk.sampler.MetropolisExchange(hi, graph=g, d_max=1, n_chains=512)
        st = sampler.init_state(model, flat, seed=17)
        a, st = sampler.sample(model, flat, state=st, chain_length=4, n_discard=5)
        out.append((a.clone(), st.log_prob.clone(), st.n_accepted_proc.clone()))
    assert torch.equal(out[0][0], out[1][0])
    assert torch.equal(out[0][1], out[1][1])
    assert torch.equal(out[0][2], out[1][2])
    assert torch.all(out[0][0].to(torch.int32).sum(-1) == 0)


def test_sampler_bookkeeping(nk):
    N = 20
    model = nk.models.RBM(alpha=2)
    flat = model.init_flat(1, N)
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    sampler = nk.sampler.MetropolisExchange(hi, graph=nk.graph.Chain(N), n_chains=128)
    s1 = sampler.init_state(model, flat, seed=5)
    a, s1 = sampler.sample(model, flat, state=s1, chain_length=7, n_discard=3)
    s2 = sampler.init_state(model, flat, seed=5)
    b, s2 = sampler.sample(model, flat, state=s2, chain_length=7, n_discard=3)
    assert a.shape == (128, 7, N)
    assert torch.equal(a, b), "same seed must give identical chains"
    assert torch.all(a.to(torch.int32).sum(-1) == 0)
    assert torch.equal(a[:, -1], s1.σ)
    lp = 2 * model.apply(flat, s1.σ)
    torch.testing.assert_close(s1.log_prob, lp, rtol=1e-12, atol=1e-12)
    assert s1.n_steps_proc == 128 * 10 * N
    acc = s1.acceptance
    assert 0.05 < acc <= 1.0
    c, s1 = sampler.sample(model, flat, state=s1, chain_length=2)
    assert not torch.equal(c[:, 0], a[:, 0])


def test_local_sampler_fp32_matches_fp64_marginals(nk):
    """FP32 and FP64 sampling of the same model agree on <x_i x_j> within error."""
    N = 16
    model = nk.models.RBM(alpha=1, kernel_init_std=0.3, hidden_bias_init_std=0.3,
                          visible_bias_init_std=0.3)
    flat = model.init_flat(3, N)
    hi = nk.hilbert.Spin(0.5, N)
    corr = []
    for dt in (torch.float64, torch.float32):
        sampler = nk.sampler.MetropolisLocal(hi, n_chains=1024)
        st = sampler.init_state(model, flat.to(dt), seed=11)
        s, st = sampler.sample(model, flat.to(dt), state=st, chain_length=64, n_discard=32)
        s = s.reshape(-1, N).to(torch.float64)
        corr.append((s[:, :-1] * s[:, 1:]).mean(0).cpu().numpy())
    assert np.all(np.abs(corr[0] - corr[1]) < 0.03)


# ------------------------------------------------------------------ Hamiltonian rule
def _plaquette_op(nk, hi, N):
    """ZZ bonds, 4-site XXXX and 3-site XZX terms and single-site X terms:
    proposals change 1 to 4 sites at once."""
    sx = np.array([[0.0, 1.0], [1.0, 0.0]])
    sz = np.array([[1.0, 0.0], [0.0, -1.0]])
    ops, aon = [], []
    for i in range(N):
        ops.append(0.8 * np.kron(sz, sz))
        aon.append([i, (i + 1) % N])
    for i in range(0, N, 2):
        ops.append(-0.6 * np.kron(np.kron(sx, sx), np.kron(sx, sx)))
        aon.append(sorted([i, (i + 1) % N, (i + 2) % N, (i + 3) % N]))
    ops.append(-0.4 * np.kron(np.kron(sx, sz), sx))
    aon.append([0, 1, 2])
    for i in range(N):  # single flips make the chain ergodic on all 2^N states
        ops.append(-0.5 * sx)
        aon.append([i])
    return nk.operator.LocalOperator(hi, ops, aon)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("std,independent", [(0.1, False), (0.5, True)])
def test_hamiltonian_rule_heisenberg_distribution(nk, dtype, std, independent):
    """Heisenberg (diagonal slot always counted): stays in the Sz = 0 sector and
    samples |psi|^2 there."""
    N = 8
    model = _model(nk, std)
    flat = model.init_flat(9, N)
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    H = nk.operator.Heisenberg(hi, nk.graph.Chain(N))
    make = lambda nc: nk.sampler.MetropolisHamiltonian(hi, H, n_chains=nc)
    assert make(1).rule.diag_rule == 1
    assert _chi2_pvalues(nk, make, model, flat, N, 0, dtype, independent=independent) > 0.01


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_hamiltonian_rule_ising_distribution(nk, dtype):
    """Ising on an open chain (diagonal slot only where J sum s_i s_j != 0)."""
    N = 7
    model = _model(nk, 0.5)
    flat = model.init_flat(10, N)
    hi = nk.hilbert.Spin(0.5, N)
    H = nk.operator.Ising(hi, nk.graph.Chain(N, pbc=False), h=0.9, J=1.1)
    make = lambda nc: nk.sampler.MetropolisHamiltonian(hi, H, n_chains=nc)
    assert make(1).rule.diag_rule == 2
    assert _chi2_pvalues(nk, make, model, flat, N, None, dtype, independent=True) > 0.01


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_hamiltonian_rule_multisite_distribution(nk, dtype):
    """4-site and 3-site off-diagonal terms.  Parameters N(0, 0.25^2) from a
    fixed numpy seed: every one of the 256 states expects >= 0.2 of the 10,240
    samples and none more than 620 (with std 0.5 one state holds 81 % of |psi|^2
    and no sampler, the oracle's included, equilibrates between the modes in 30
    sweeps)."""
    N = 8
    model = _model(nk, 0.5)
    M = model.n_hidden(N)
    flat = torch.as_tensor(np.random.default_rng(11).normal(0, 0.25, M + N * M + N),
                           device="cuda")
    hi = nk.hilbert.Spin(0.5, N)
    H = _plaquette_op(nk, hi, N)
    make = lambda nc: nk.sampler.MetropolisHamiltonian(hi, H, n_chains=nc)
    assert _chi2_pvalues(nk, make, model, flat, N, None, dtype, independent=True) > 0.01


def test_hamiltonian_rule_matches_oracle_acceptance(nk):
    """Mean acceptance per proposal agrees with the oracle's numba-form rule
    run on the same initial states (both are exact Metropolis chains, so their
    stationary acceptance rates agree within sampling error)."""
    from gpu_common import oracle_local
    from oracle import sampler as osamp
    N = 8
    model = _model(nk, 0.4)
    flat = model.init_flat(12, N)
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    H = nk.operator.Heisenberg(hi, nk.graph.Chain(N, max_neighbor_order=2), J=[1.0, 0.5])
    sampler = nk.sampler.MetropolisHamiltonian(hi, H, n_chains=2048)
    st = sampler.init_state(model, flat, seed=4)
    _, st = sampler.sample(model, flat, state=st, chain_length=1, n_discard=20)
    st = sampler.reset(model, flat, st)
    x0 = st.σ.clone()
    _, st = sampler.sample(model, flat, state=st, chain_length=5)
    acc_gpu = st.acceptance
    rng = np.random.default_rng(0)
    p = oracle_params(flat, N, model.n_hidden(N))
    _, _, _, nacc = osamp.sample_chain(p, x0[:512].cpu().numpy(), rng, 5, rule="hamiltonian",
                                       operator=oracle_local(H), diag_rule=1)
    acc_or = nacc.sum() / (512 * 5 * N)
    sd = np.sqrt(acc_or * (1 - acc_or) / (512 * 5 * N)) * 4  # correlated proposals: x4
    assert abs(acc_gpu - acc_or) < max(4 * sd, 0.01), (acc_gpu, acc_or)


def test_hamiltonian_rule_bookkeeping(nk):
    N = 16
    model = nk.models.RBM(alpha=2)
    flat = model.init_flat(3, N)
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    H = nk.operator.Heisenberg(hi, nk.graph.Chain(N))
    sampler = nk.sampler.MetropolisHamiltonian(hi, H, n_chains=256)
    s1 = sampler.init_state(model, flat, seed=5)
    a, s1 = sampler.sample(model, flat, state=s1, chain_length=6, n_discard=4)
    s2 = sampler.init_state(model, flat, seed=5)
    b, s2 = sampler.sample(model, flat, state=s2, chain_length=6, n_discard=4)
    assert torch.equal(a, b)
    assert torch.all(a.to(torch.int32).sum(-1) == 0), "Sz must be conserved"
    assert torch.equal(a[:, -1], s1.σ)
    torch.testing.assert_close(s1.log_prob, 2 * model.apply(flat, s1.σ), rtol=1e-12, atol=1e-12)
    assert int(sampler.rule.status.item()) == 0
    assert 0.05 < s1.acceptance <= 1.0
    with pytest.raises(ValueError, match="hilbert"):
        nk.sampler.MetropolisHamiltonian(nk.hilbert.Spin(0.5, N), H, n_chains=4)
    with pytest.raises(TypeError):
        nk.sampler.MetropolisHamiltonian(hi, "not an operator")


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_hamiltonian_rule_pauli_distribution(nk, dtype):
    """PauliStrings operator: XX+YY exchange (zero on aligned pairs, so n(x)
    varies), ZZ, a 4-site XXXX string and single X strings."""
    N = 8
    hi = nk.hilbert.Spin(0.5, N)
    ops, w = [], []
    for i in range(N):
        j = (i + 1) % N
        for c, wc in (("X", 0.5), ("Y", 0.5), ("Z", 1.0)):
            s = ["I"] * N
            s[i] = s[j] = c
            ops.append("".join(s))
            w.append(wc)
        s = ["I"] * N
        s[i] = "X"
        ops.append("".join(s))
        w.append(-0.3)
    ops.append("XXXXIIII")
    w.append(0.4)
    H = nk.operator.PauliStrings(hi, ops, w)
    model = _model(nk, 0.5)
    M = model.n_hidden(N)
    flat = torch.as_tensor(np.random.default_rng(11).normal(0, 0.25, M + N * M + N),
                           device="cuda")
    make = lambda nc: nk.sampler.MetropolisHamiltonian(hi, H, n_chains=nc)
    assert _chi2_pvalues(nk, make, model, flat, N, None, dtype, independent=True) > 0.01
    s = make(64)
    st = s.init_state(model, flat.to(dtype), seed=1)
    _, st = s.sample(model, flat.to(dtype), state=st, chain_length=3)
    assert int(s.rule.status.item()) == 0


def test_hamiltonian_rule_pauli_sz_conserving(nk):
    """XX + YY + ZZ strings conserve Sz: chains started at Sz = 0 stay there,
    and the acceptance agrees with the oracle's rule."""
    from oracle import sampler as osamp
    N = 10
    hi = nk.hilbert.Spin(0.5, N, total_sz=0)
    ops, w = [], []
    for i in range(N):
        for c, wc in (("X", 1.0), ("Y", 1.0), ("Z", 1.0)):
            s = ["I"] * N
            s[i] = s[(i + 1) % N] = c
            ops.append("".join(s))
            w.append(wc)
    H = nk.operator.PauliStrings(hi, ops, w)
    model = _model(nk, 0.3)
    flat = model.init_flat(2, N)
    sampler = nk.sampler.MetropolisHamiltonian(hi, H, n_chains=1024)
    st = sampler.init_state(model, flat, seed=3)
    a, st = sampler.sample(model, flat, state=st, chain_length=4, n_discard=10)
    assert torch.all(a.to(torch.int32).sum(-1) == 0)
    torch.testing.assert_close(st.log_prob, 2 * model.apply(flat, st.σ), rtol=1e-12, atol=1e-12)
    st = sampler.reset(model, flat, st)
    x0 = st.σ[:512].cpu().numpy().copy()
    _, st = sampler.sample(model, flat, state=st, chain_length=4)
    p = oracle_params(flat, N, model.n_hidden(N))
    rng = np.random.default_rng(5)
    x, acc = x0, 0
    lp = 2 * orbm.logpsi(p, x)
    for _ in range(4 * N):
        xp, corr = osamp.pauli_hamiltonian_propose(ops, w, x, rng.random(len(x)))
        lpp = 2 * orbm.logpsi(p, xp)
        ok = rng.random(len(x)) < np.exp(lpp - lp + corr)
        x = np.where(ok[:, None], xp, x)
        lp = np.where(ok, lpp, lp)
        acc += ok.sum()
    acc_or = acc / (512 * 4 * N)
    assert abs(st.acceptance - acc_or) < 0.03, (st.acceptance, acc_or)


def test_reset_chains(nk):
    """reset_chains=True (netket/sampler/metropolis.py:382-414): every reset
    restarts the chains from fresh random states (a new Philox stream per
    reset) and recomputes log_prob; without it the chains continue."""
    N = 12
    hi = nk.hilbert.Spin(0.5, N)
    model = nk.models.RBM(alpha=1)
    flat = model.init_flat(2, N)
    s = nk.sampler.MetropolisLocal(hi, n_chains=64, reset_chains=True)
    st = s.init_state(model, flat, seed=9)
    a, st = s.sample(model, flat, state=st, chain_length=3)
    c0 = st.counter
    st = s.reset(model, flat, st)
    assert torch.equal(st.σ, hi.random_state(st.seed, 64, stream_id=2 + c0))
    assert not torch.equal(st.σ, a[:, -1])
    torch.testing.assert_close(st.log_prob, 2 * model.apply(flat, st.σ), rtol=1e-12, atol=1e-12)
    b, st = s.sample(model, flat, state=st, chain_length=3)
    assert not torch.equal(s.reset(model, flat, st).σ, b[:, -1])
    s2 = nk.sampler.MetropolisLocal(hi, n_chains=64)
    st2 = s2.init_state(model, flat, seed=9)
    c, st2 = s2.sample(model, flat, state=st2, chain_length=3)
    assert torch.equal(s2.reset(model, flat, st2).σ, c[:, -1])

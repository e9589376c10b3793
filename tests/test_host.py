"""CPU tests of the product's host side: lattice edges, operator packing, the
C-ABI library (loads and exports every declared symbol), and loud failure
without a GPU.  No kernel is launched here."""
import math
import os
import re

import numpy as np
import pytest
import torch

from oracle import hilbert as oh
from oracle import operator as oop

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="session")
def built_lib():
    from netket_gb300 import build
    return build.build()


def test_philox_known_answers():
    """Random123 known-answer vectors for Philox4x32-10."""
    from philox_ref import philox4x32_10
    assert philox4x32_10((0, 0, 0, 0), (0, 0)) == (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    F = 0xFFFFFFFF
    assert philox4x32_10((F, F, F, F), (F, F)) == (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)
    assert philox4x32_10((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344),
                         (0xA4093822, 0x299F31D0)) == (0xD16CFE09, 0x94FDCCEB, 0x5001E420,
                                                       0x24126EA1)


@pytest.mark.parametrize("name", ["chain16", "chain5", "chain8_obc", "chain14_nnn", "square4",
                                  "square6_nnn", "square10_nnn", "square16", "cube3"])
def test_product_lattice_edges_match_reference(golden, name):
    from netket_gb300 import graph
    g = golden("edges")
    meta = g[name + "__meta"]
    L = graph.Grid(list(meta[:-2]), pbc=bool(meta[-2]), max_neighbor_order=int(meta[-1]))
    np.testing.assert_array_equal(np.array(L.edges(return_color=True)).reshape(-1, 3), g[name])


def test_graph_distances_and_bipartite():
    from netket_gb300 import graph
    g = graph.Chain(6)
    d = g.distances()
    assert d[0, 3] == 3 and d[0, 5] == 1
    assert g.is_bipartite() and not graph.Chain(5).is_bipartite()
    assert not graph.Square(4, max_neighbor_order=2).is_bipartite()


LOCALOP_CASES = ["heis_chain16", "heis_square4", "heis_square4_nosign", "j1j2_square6",
                 "j1j2_chain14", "j1j2_square10", "ising_local_chain5"]


@pytest.mark.parametrize("name", LOCALOP_CASES)
def test_product_packing_matches_reference(golden, name):
    """The device tables reproduce the reference packer's max_conn_size and the
    oracle's term order / connections (checked on the host copy of the tables)."""
    from netket_gb300 import hilbert, operator
    gl = golden("localop")
    N = int(gl[name + "__N"])
    ops, aon = [], []
    for a, m, s in zip(gl[name + "__aon"], gl[name + "__ops"], gl[name + "__sizes"]):
        d = 2**int(s)
        ops.append(m[:d, :d])
        aon.append([int(v) for v in a[:s]])
    op = operator.LocalOperator(hilbert.Spin(0.5, N), ops, aon)
    assert op.max_conn_size == int(gl[name + "__max_conn_jax"])
    ref = oop.LocalOperator(N, ops, aon)
    tb = op._pack()
    # emulate the device enumeration on the host tables for a few samples
    x = oh.local_indices_to_states(gl[name + "__x_ids"])[:5]
    rxp, rm = ref.get_conn_padded(x)
    for b in range(len(x)):
        cand = []
        rows = []
        for t in range(tb["T"]):
            sz = tb["acting_size"][t]
            r = 0
            for q in range(sz):
                r = (r << 1) | int(x[b, tb["acting_on"][t, q]] < 0)
            rows.append(r)
        if tb["nonzero_diag"]:
            tot, t = 0.0, 0
            for ge in tb["group_end"]:
                gs = 0.0
                while t < ge:
                    gs += tb["diag"][t, rows[t]]
                    t += 1
                tot += gs
            d = 0.0 + tot
            if abs(d) > 1e-10:
                cand.append(d)
        for t in range(tb["T"]):
            for c in range(tb["n_conns"][t, rows[t]]):
                cand.append(tb["mels"][t, rows[t], c])
        K = tb["K"]
        got = np.zeros(K)
        got[:len(cand)] = cand
        np.testing.assert_array_equal(got, rm[b])


def test_header_symbols_exported(built_lib):
    """Every entry point declared in include/vmck.h is exported by libvmck.so and
    has a ctypes signature."""
    import ctypes
    from netket_gb300 import _native
    hdr = open(os.path.join(ROOT, "include", "vmck.h")).read()
    declared = set(re.findall(r"\b(vmck_[a-z0-9_]+)\s*\(", hdr))
    lib = ctypes.CDLL(built_lib)
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(_native.declared_symbols())
    L = _native.lib()
    assert L.vmck_abi_version() == 1
    assert L.vmck_error_string(1) == b"invalid argument"


def test_argument_errors_are_reported(built_lib):
    """Host-side argument checks return an error code without touching a GPU."""
    from netket_gb300 import _native
    L = _native.lib()
    rc = L.vmck_get_conn_ising(None, None, 4, 8, None, 0, 1.0, 1.0, 0, None, None, None)
    assert rc == 1 and b"argument" in L.vmck_last_error()
    assert L.vmck_stats_workspace_size(16, 63) == 3 * 16 + 16 * (63 // 1)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU behaviour")
def test_fails_loudly_without_gpu(built_lib):
    import netket_gb300 as nk
    hi = nk.hilbert.Spin(0.5, N=4)
    with pytest.raises(nk._native.VmckError):
        hi.random_state(0, 3)


def test_state_dict_bytes_round_trip():
    """The checkpoint byte format keeps NetKet's nested state-dict structure and
    every array bit for bit (uint64 rng words, int8 chains, FP64 parameters)."""
    from netket_gb300 import serialization as ser
    rng = np.random.default_rng(0)
    d = {"variables": {"params": {"Dense": {"bias": rng.normal(size=4),
                                            "kernel": rng.normal(size=(3, 4))},
                                  "visible_bias": rng.normal(size=3)}},
         "sampler_state": {"σ": rng.choice(np.array([-1, 1], dtype=np.int8), size=(5, 3)),
                           "rng": np.array([2**64 - 1, 12345], dtype=np.uint64),
                           "n_steps_proc": np.int64(7), "n_accepted_proc": np.arange(5)},
         "n_samples": np.int64(20), "n_discard_per_chain": np.int64(5)}
    back = ser.dict_from_bytes(ser.dict_to_bytes(d))

    def check(a, b):
        if isinstance(a, dict):
            assert set(a) == set(b)
            for k in a:
                check(a[k], b[k])
        else:
            assert np.asarray(a).dtype == np.asarray(b).dtype
            np.testing.assert_array_equal(a, b)
    check(d, back)


def _online_from_oracle(s, decay=None, device="cpu"):
    from netket_gb300.online_stats import OnlineStats
    d = {k: s[k] for k in ("count", "mean", "M2", "cross", "m1", "m2", "pair", "buf")}
    d.update(max_lag=s["max_lag"], n_total=s["n_total"], buf_len=s["buf_len"],
             decay=-1.0 if decay is None else decay)
    return OnlineStats.from_state_dict(d, device=device)


@pytest.mark.parametrize("name", ["iid_oneshot", "iid_chunks", "ar1_small_batches",
                                  "ar1_ragged", "big_then_small", "decay", "no_acf",
                                  "one_chain", "shifted_mean"])
def test_online_stats_readouts(golden, name):
    """OnlineStats read-outs (mean, variance, tau via Geyer / batch, R-hat, error,
    ACF) on the accumulator state, vs the reference's own read-outs."""
    from test_oracle_golden import acf_tolerance, online_oracle_run
    g = golden("online_stats")
    cfg = g[name + "__cfg"]
    est = _online_from_oracle(online_oracle_run(g, name), None if cfg[1] < 0 else cfg[1])
    st = est.get_stats()
    got = np.array([est.mean, est.variance, est.tau_corr, est.tau_corr_batch, est.tau_corr_acf,
                    est.R_hat, st.error_of_mean])
    np.testing.assert_allclose(got, g[name + "__derived"], rtol=1e-11, atol=1e-13,
                               equal_nan=True)
    assert st.mean == est.mean and st.tau_corr == est.tau_corr
    ga = g[name + "__acf"]
    if ga.size == 0:
        assert est.acf is None
    else:
        np.testing.assert_allclose(est.acf.numpy(), ga, rtol=0, atol=acf_tolerance(g, name))
    key, d = est.to_compound()
    assert key == "Mean" and set(d) >= {"Mean", "Variance", "Sigma", "R_hat", "TauCorr"}


def test_online_stats_window_operations():
    """expand_max_lag / thin_acf_by_2 (netket/_src/stats/online_stats/
    operations.py:129-261), the reference tests' properties: old lags kept, new
    lags zero, buffer right-aligned, Welford state untouched, even lags kept."""
    from oracle import online_stats as oos
    from netket_gb300.online_stats import expand_max_lag, thin_acf_by_2
    rng = np.random.default_rng(5)
    s = oos.new_state(4, 16)
    for ch in np.split(rng.standard_normal((4, 200)), 4, axis=1):
        s = oos.update(s, ch)
    est = _online_from_oracle(s)
    ex = expand_max_lag(est, 48)
    assert ex.max_lag == 48 and ex._cross_sum.shape == (4, 49) and ex._chain_buf.shape == (4, 48)
    np.testing.assert_array_equal(ex._cross_sum[:, :17].numpy(), s["cross"])
    np.testing.assert_array_equal(ex._pair_count[:, :17].numpy(), s["pair"])
    assert not ex._cross_sum[:, 17:].any() and not ex._pair_count[:, 17:].any()
    np.testing.assert_array_equal(ex._chain_buf[:, 32:].numpy(), s["buf"])
    assert not ex._chain_buf[:, :32].any()
    np.testing.assert_array_equal(est.acf.numpy(), ex.acf[:17].numpy())
    assert ex.mean == est.mean and ex.variance == est.variance and ex.n_samples == est.n_samples
    with pytest.raises(ValueError, match="must be >"):
        expand_max_lag(est, 16)
    th = thin_acf_by_2(est)
    assert th.max_lag == 8 and th._buf_len == s["buf_len"] // 2
    np.testing.assert_array_equal(th._cross_sum.numpy(), s["cross"][:, ::2])
    np.testing.assert_array_equal(th._chain_buf.numpy(), s["buf"][:, 0::2])
    z = _online_from_oracle(oos.update(oos.new_state(4, 0), rng.standard_normal((4, 10))))
    assert z.acf is None and math.isnan(z.tau_corr_acf)
    ez = expand_max_lag(z, 32)
    assert ez._cross_sum.shape == (4, 33) and ez._chain_buf.shape == (4, 32)


def test_online_stats_batch_delta_method():
    """OnlineStatsBatch: combinator of K channel means with the delta-method
    error J^T Cov J, Cov the covariance of the chain means / n_chains
    (accumulator_batch.py:31-68, 196-211)."""
    from oracle import online_stats as oos
    from netket_gb300.online_stats import OnlineStatsBatch
    rng = np.random.default_rng(8)
    data = rng.standard_normal((64, 50, 2)) + np.array([0.5, 1.0])
    ests = []
    for k in range(2):
        ests.append(_online_from_oracle(oos.update(oos.new_state(64, 8), data[..., k])))
    acc = OnlineStatsBatch(ests, lambda mu: mu[1] - mu[0] ** 2)
    X = data.reshape(-1, 2).mean(0)
    cm = data.mean(1)
    cov = (cm - X).T @ (cm - X) / 64 ** 2
    J = np.array([-2 * X[0], 1.0])
    st = acc.get_stats()
    np.testing.assert_allclose(st.mean, X[1] - X[0] ** 2, rtol=1e-12)
    np.testing.assert_allclose(st.error_of_mean, np.sqrt(J @ cov @ J), rtol=1e-10)
    vec = OnlineStatsBatch(ests, lambda mu: torch.stack([mu[0], mu[0] * mu[1]])).get_stats()
    assert tuple(vec.mean.shape) == (2,) and tuple(vec.error_of_mean.shape) == (2,)
    np.testing.assert_allclose(float(vec.error_of_mean[0]), np.sqrt(cov[0, 0]), rtol=1e-10)


def test_pauli_strings_pack_matches_oracle(golden):
    """Host packer of PauliStrings: slot order, flip sites, string weights with
    the (-i)^#Y factor and Z-check sites equal the oracle's grouping (which is
    pinned to the reference's pack_internals_jax)."""
    from oracle import operator as oop_
    import netket_gb300 as nk
    g = golden("pauli_strings")
    for name in ("tfim", "heisenberg_xyz", "mixed", "duplicates_and_zeros"):
        ops, w = list(g[name + "__raw_ops"]), g[name + "__raw_weights"]
        N = len(ops[0])
        op = nk.operator.PauliStrings(nk.hilbert.Spin(0.5, N), ops, w)
        assert op.operators == list(g[name + "__ops"])
        np.testing.assert_array_equal(op.weights, g[name + "__weights"])
        tb = op._pack()
        ref = oop_.pauli_pack(g[name + "__ops"], g[name + "__weights"])
        assert tb["F"] == len(ref)
        for f, (flip, rest) in enumerate(ref):
            sites = tb["flip_site"][tb["flip_offset"][f]:tb["flip_offset"][f + 1]]
            assert tuple(sites) == flip
            bits = [i for i in range(N) if (tb["flip_mask"][f, i // 32] >> (i % 32)) & 1]
            assert tuple(bits) == flip
            s0, s1 = tb["string_offset"][f], tb["string_offset"][f + 1]
            assert s1 - s0 == len(rest)
            for k, (wt, z) in enumerate(rest):
                assert tb["weight"][s0 + k] == wt
                zs = [i for i in range(N) if (tb["z_mask"][s0 + k, i // 32] >> (i % 32)) & 1]
                assert zs == z
    hi = nk.hilbert.Spin(0.5, 3)
    with pytest.raises(TypeError):
        nk.operator.PauliStrings(hi, ["YII"], [1.0])
    with pytest.raises(ValueError):
        nk.operator.PauliStrings(hi, ["XQI"], [1.0])


def _header_prototypes():
    """{name: (return kind, [argument kinds])} parsed from include/vmck.h."""
    hdr = open(os.path.join(ROOT, "include", "vmck.h")).read()
    hdr = re.sub(r"/\*.*?\*/", " ", hdr, flags=re.S)
    protos = {}
    for ret, name, args in re.findall(
            r"\b(uint64_t|int64_t|int|const\s+char\s*\*)\s*(vmck_[a-z0-9_]+)\s*\(([^)]*)\)\s*;",
            hdr):
        kinds = []
        for a in args.split(","):
            a = a.strip()
            if not a or a == "void":
                continue
            if "*" in a or a.startswith("vmck_stream"):
                kinds.append("ptr")
            elif re.match(r"(const\s+)?uint64_t\b", a):
                kinds.append("u64")
            elif re.match(r"(const\s+)?int64_t\b", a):
                kinds.append("i64")
            elif re.match(r"(const\s+)?(int32_t|int)\b", a):
                kinds.append("i32")
            elif re.match(r"(const\s+)?double\b", a):
                kinds.append("f64")
            else:
                raise AssertionError(f"{name}: unclassified argument {a!r}")
        rk = {"int": "i32", "int64_t": "i64", "uint64_t": "u64"}.get(ret, "str")
        protos[name] = (rk, kinds)
    return protos


def test_ctypes_signatures_match_header():
    """Every ctypes binding has the header prototype's argument count, kinds
    (pointer / int32 / int64 / uint64 / double) and return type."""
    import ctypes
    from netket_gb300 import _native

    def kind(t):
        if t in (ctypes.c_void_p, ctypes.c_char_p) or hasattr(t, "_type_") and \
                isinstance(getattr(t, "_type_"), type):
            return "ptr"
        return {ctypes.c_int32: "i32", ctypes.c_int64: "i64", ctypes.c_uint64: "u64",
                ctypes.c_double: "f64"}[t]

    protos = _header_prototypes()
    assert set(protos) == set(_native.declared_symbols())
    for name, (args, res) in _native._SIGNATURES.items():
        rk, kinds = protos[name]
        assert [kind(a) for a in args] == kinds, name
        exp_res = {"i32": ctypes.c_int32, "i64": ctypes.c_int64, "u64": ctypes.c_uint64,
                   "str": ctypes.c_char_p}[rk]
        assert res is exp_res, name


def test_expect_to_precision_stopping_rule():
    """``not_converged`` is _check_not_converged of expect_to_precision.py:26-41:
    absolute and relative tests with '>', 0 / inf relative error at zero mean,
    NaN errors stop."""
    from netket_gb300.online_stats import not_converged
    from netket_gb300.stats import Stats
    nan = float("nan")
    assert not_converged(Stats(mean=1.0, error_of_mean=0.2), 0.1, None)
    assert not not_converged(Stats(mean=1.0, error_of_mean=0.1), 0.1, None)
    assert not_converged(Stats(mean=2.0, error_of_mean=0.1), None, 0.01)
    assert not not_converged(Stats(mean=-20.0, error_of_mean=0.1), None, 0.01)
    assert not_converged(Stats(mean=-20.0, error_of_mean=0.1), 0.05, 0.01)  # both must hold
    assert not_converged(Stats(mean=0.0, error_of_mean=1e-9), None, 0.5)    # inf relative
    assert not not_converged(Stats(mean=0.0, error_of_mean=0.0), None, 0.5)
    assert not not_converged(Stats(mean=1.0, error_of_mean=nan), 0.1, 0.1)


C_CALLER = r"""
#include <stdio.h>
#include <string.h>
#include "vmck.h"

/* A C caller of the ABI (what a cgo / C FFI binding would compile): entry
   points that need no GPU -- version, error strings, argument checks. */
int main(void) {
  if (vmck_abi_version() != VMCK_ABI_VERSION) return 10;
  if (strcmp(vmck_error_string(VMCK_ERR_ARG), "invalid argument") != 0) return 11;
  if (vmck_get_conn_ising(NULL, NULL, 4, 8, NULL, 0, 1.0, 1.0, 0, NULL, NULL, NULL)
      != VMCK_ERR_ARG) return 12;
  if (vmck_online_stats_update(NULL, NULL, 4, 2, 8, 0, 1.0, 0, NULL) != VMCK_ERR_ARG) return 13;
  vmck_pauli_strings ps;
  memset(&ps, 0, sizeof ps);
  if (vmck_get_conn_pauli(NULL, &ps, NULL, 1, NULL, NULL, NULL) != VMCK_ERR_ARG) return 14;
  if (vmck_stats_workspace_size(16, 63) != 3 * 16 + 16 * 63) return 15;
  printf("%s\n", vmck_last_error());
  return 0;
}
"""


def test_c_caller_compiles_and_links(built_lib, tmp_path):
    """include/vmck.h is valid C99 and libvmck.so is callable from C."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(built_lib)
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-pedantic", str(src),
                        "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lvmck",
                        "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.strip()  # the last argument error's message


def test_exchange_rule_arguments():
    """ExchangeRule (netket/sampler/rules/exchange.py:100-142, 190-205): clusters
    from graph distances (i < j), exactly one of clusters / graph, positive
    probabilities; uniform probabilities are the default rule, non-uniform ones
    are refused."""
    import netket_gb300 as nk
    g = nk.graph.Chain(6, max_neighbor_order=2)
    r = nk.sampler.ExchangeRule(graph=g, d_max=1)
    assert len(r.clusters) == 12 and np.all(r.clusters[:, 0] < r.clusters[:, 1])
    assert len(nk.sampler.ExchangeRule(graph=nk.graph.Chain(6), d_max=2).clusters) == 12
    assert len(nk.sampler.ExchangeRule(graph=g, probabilities=[2.0, 2.0]).clusters) == 12
    with pytest.raises(ValueError):
        nk.sampler.ExchangeRule()
    with pytest.raises(ValueError):
        nk.sampler.ExchangeRule(graph=g, clusters=[(0, 1)])
    with pytest.raises(ValueError, match="positive"):
        nk.sampler.ExchangeRule(graph=g, probabilities=[1.0, -1.0])
    with pytest.raises(NotImplementedError):
        nk.sampler.ExchangeRule(graph=g, probabilities=[1.0, 0.5])


def test_driver_and_state_arguments_refused_before_the_device():
    """NetKet's MCState / VMC_SR arguments outside this path are refused with a
    clear error (checked before any device work)."""
    import netket_gb300 as nk
    hi = nk.hilbert.Spin(0.5, 4)
    sa = nk.sampler.MetropolisLocal(hi, n_chains=4)
    with pytest.raises(NotImplementedError, match="init_fun"):
        nk.vqs.MCState(sa, nk.models.RBM(), init_fun=lambda *a: None)
    with pytest.raises(NotImplementedError, match="mutable"):
        nk.vqs.MCState(sa, nk.models.RBM(), mutable=True)
    H = nk.operator.Ising(hi, nk.graph.Chain(4), h=1.0)
    opt = nk.optimizer.Sgd(0.01)
    with pytest.raises(NotImplementedError, match="linear_solver"):
        nk.driver.VMC_SR(H, opt, diag_shift=0.01, variational_state=None,
                         linear_solver=lambda A, b: (b, None))
    with pytest.raises(NotImplementedError, match="mode"):
        nk.driver.VMC_SR(H, opt, diag_shift=0.01, variational_state=None, mode="complex")
    with pytest.raises(NotImplementedError, match="on_the_fly"):
        nk.driver.VMC_SR(H, opt, diag_shift=0.01, variational_state=None, use_ntk=False,
                         on_the_fly=True)
    # linear_solver_fn: the reference's deprecated name for linear_solver
    with pytest.warns(FutureWarning, match="linear_solver_fn"):
        with pytest.raises(NotImplementedError, match="linear_solver"):
            nk.driver.VMC_SR(H, opt, diag_shift=0.01, variational_state=None,
                             linear_solver_fn=lambda A, b: (b, None))
    with pytest.raises(ValueError, match="linear_solver only"):
        nk.driver.VMC_SR(H, opt, diag_shift=0.01, variational_state=None,
                         linear_solver=nk.optimizer.solver.cholesky,
                         linear_solver_fn=nk.optimizer.solver.cholesky)


def _replica_rank(rank, world, port, q):
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        ms = [12.5, 20.0][rank]  # the second replica is the slow one
        ms_max = bench.max_over_ranks(ms, dist, "cpu")
        q.put((rank, ms_max, bench.replica_throughput(world, ms_max)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_timing_two_ranks_gloo():
    """bench.py's N > 1 path (replicas only): every rank sees the slowest
    replica's time, and the whole-job throughput is world x 1000 / that time;
    2 ranks on the gloo backend."""
    import socket
    import torch.multiprocessing as mp
    import bench
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [20.0, 20.0]
    assert all(abs(r[2] - 2 * 1000.0 / 20.0) < 1e-12 for r in res)
    assert bench.max_over_ranks(7.25) == 7.25 and bench.replica_throughput(1, 25.0) == 40.0


def test_pauli_strings_algebra():
    """PauliStrings +, -, scalar + and * (netket/operator/_pauli_strings/base.py:
    373-470): sums concatenate and reduce like the constructor, scalars add the
    identity string, * scales the weights; the tables equal the oracle's."""
    from oracle import operator as oop_
    import netket_gb300 as nk
    hi = nk.hilbert.Spin(0.5, 4)
    A = nk.operator.PauliStrings(hi, ["XXII", "ZZII"], [0.5, 1.0])
    B = nk.operator.PauliStrings(hi, ["ZZII", "IYYI"], [0.25, 2.0])
    C = A + B
    ops, w = oop_.pauli_canonicalize(["XXII", "ZZII", "ZZII", "IYYI"], [0.5, 1.0, 0.25, 2.0])
    assert C.operators == list(ops) and C.weights == list(w)
    D = 2.0 * A - B
    ops, w = oop_.pauli_canonicalize(["XXII", "ZZII", "ZZII", "IYYI"], [1.0, 2.0, -0.25, -2.0])
    assert D.operators == list(ops) and np.allclose(D.weights, w)
    E = A + 3.0
    assert "IIII" in E.operators and E.weights[E.operators.index("IIII")] == 3.0
    assert (A * 0.5).weights == [0.25, 0.5] and (A * 0.5).operators == A.operators
    assert (-A).weights == [-0.5, -1.0]
    tb, ref = D._pack(), oop_.pauli_pack(*oop_.pauli_canonicalize(D.operators, D.weights))
    assert tb["F"] == len(ref)
    with pytest.raises(TypeError):
        A * B
    with pytest.raises(ValueError):
        A + nk.operator.PauliStrings(nk.hilbert.Spin(0.5, 4, total_sz=0), ["XXII"], [1.0])


def _dense_from_local(N, terms, constant):
    """Dense H from (sites, matrix) terms; basis index = sum idx(x_i) 2^(N-1-i),
    idx(+1) = 0; a term's row index takes its first site as the leading bit."""
    dim = 2 ** N
    H = constant * np.eye(dim)
    for aon, m in terms:
        k = len(aon)
        for col in range(dim):
            bits = [(col >> (N - 1 - i)) & 1 for i in range(N)]
            c = sum(bits[s] << (k - 1 - q) for q, s in enumerate(aon))
            for r in range(2 ** k):
                if m[r, c] == 0:
                    continue
                nb = list(bits)
                for q, s in enumerate(aon):
                    nb[s] = (r >> (k - 1 - q)) & 1
                row = sum(b << (N - 1 - i) for i, b in enumerate(nb))
                H[row, col] += m[r, c]
    return H


def _dense_from_pauli(N, strings, weights):
    basis = {"I": np.eye(2), "X": np.array([[0.0, 1.0], [1.0, 0.0]]),
             "Y": np.array([[0.0, -1.0j], [1.0j, 0.0]]), "Z": np.diag([1.0, -1.0])}
    H = np.zeros((2 ** N, 2 ** N), dtype=complex)
    for s, w in zip(strings, weights):
        P = basis[s[0]]
        for c in s[1:]:
            P = np.kron(P, basis[c])
        H += w * P
    return H


def test_local_operator_to_pauli_strings():
    """LocalOperator.to_pauli_strings (netket/operator/_local_operator/convert.py:
    157-209) represents the same matrix: Heisenberg with the sign rule, Ising,
    and a 3-site term with a constant."""
    import netket_gb300 as nk
    N = 4
    hi = nk.hilbert.Spin(0.5, N)
    g = nk.graph.Chain(N)
    sx = np.array([[0.0, 1.0], [1.0, 0.0]])
    sz = np.diag([1.0, -1.0])
    extra = nk.operator.LocalOperator(hi, [0.7 * np.kron(np.kron(sx, sz), sx)], [[0, 2, 3]],
                                      constant=-1.5)
    for op in (nk.operator.Heisenberg(hi, g), nk.operator.Ising(hi, g, h=0.6, J=1.3)
               .to_local_operator(), extra):
        ps = op.to_pauli_strings()
        assert all(s.count("Y") % 2 == 0 for s in ps.operators)
        assert ps.operators == sorted(ps.operators) or len(set(ps.operators)) == len(ps.operators)
        H1 = _dense_from_local(N, list(op._terms.items()), op.constant)
        H2 = _dense_from_pauli(N, ps.operators, ps.weights)
        np.testing.assert_allclose(H2.imag, 0, atol=1e-12)
        np.testing.assert_allclose(H2.real, H1, atol=1e-12)


def test_local_operator_products_and_spin_helpers():
    """nk.operator.spin (netket/operator/spin.py) and LocalOperator @
    (local_operator/base.py:392-440) on dense matrices; the product's term order
    is b * A's terms, then a * B's, then the A_i B_j products."""
    import netket_gb300 as nk
    N = 4
    hi = nk.hilbert.Spin(0.5, N)
    sp = nk.operator.spin

    def dense(op):
        return _dense_from_local(N, list(op._terms.items()), op.constant)

    X = np.array([[0.0, 1.0], [1.0, 0.0]])
    Z = np.diag([1.0, -1.0])
    Y = np.array([[0.0, -1.0j], [1.0j, 0.0]])

    def on(site_mats):
        m = np.eye(1)
        for i in range(N):
            m = np.kron(m, site_mats.get(i, np.eye(2)))
        return m

    np.testing.assert_array_equal(dense(sp.sigmax(hi, 1)), on({1: X}))
    np.testing.assert_array_equal(dense(sp.sigmaz(hi, 3)), on({3: Z}))
    np.testing.assert_array_equal(dense(sp.sigmap(hi, 0)), on({0: (X + 1j * Y).real / 2}))
    np.testing.assert_array_equal(dense(sp.sigmam(hi, 2)), on({2: (X - 1j * Y).real / 2}))
    np.testing.assert_array_equal(dense(sp.identity(hi)), np.eye(2 ** N))
    with pytest.raises(TypeError):
        sp.sigmay(hi, 0)
    np.testing.assert_allclose(dense(sp.sigmaz(hi, 0) @ sp.sigmaz(hi, 2)), on({0: Z, 2: Z}))
    yy = -1.0 * ((sp.sigmap(hi, 1) - sp.sigmam(hi, 1)) @ (sp.sigmap(hi, 3) - sp.sigmam(hi, 3)))
    np.testing.assert_allclose(dense(yy), on({1: Y, 3: Y}).real, atol=1e-15)
    A = sp.sigmax(hi, 0) + 0.5
    B = sp.sigmaz(hi, 2) - 1.0 + 2.0 * (sp.sigmax(hi, 0) @ sp.sigmax(hi, 1))
    np.testing.assert_allclose(dense(A @ B), dense(A) @ dense(B), atol=1e-14)
    np.testing.assert_allclose(dense(A * B), dense(A) @ dense(B), atol=1e-14)
    H = nk.operator.Heisenberg(hi, nk.graph.Chain(N))
    np.testing.assert_allclose(dense(H @ H), dense(H) @ dense(H), atol=1e-12)
    assert list((A @ B)._terms) == [(0,), (2,), (0, 1), (0, 2)]
    assert not (sp.sigmax(hi, 0) * 0.0)._terms


def test_is_hermitian():
    """LocalOperator.is_hermitian checks its terms; the operators of the path
    (Heisenberg, J1-J2, Ising, products of Pauli matrices) are hermitian."""
    import netket_gb300 as nk
    hi = nk.hilbert.Spin(0.5, 6)
    sp = nk.operator.spin
    g = nk.graph.Chain(6, max_neighbor_order=2)
    assert nk.operator.Heisenberg(hi, nk.graph.Chain(6)).is_hermitian is True
    assert nk.operator.Heisenberg(hi, g, J=[1.0, 0.5]).is_hermitian is True
    assert nk.operator.Ising(hi, nk.graph.Chain(6), h=1.0).to_local_operator().is_hermitian
    assert nk.operator.Ising(hi, nk.graph.Chain(6), h=1.0).is_hermitian
    assert (sp.sigmaz(hi, 0) @ sp.sigmax(hi, 3)).is_hermitian
    assert (sp.sigmap(hi, 1) + sp.sigmam(hi, 1)).is_hermitian
    assert sp.sigmap(hi, 1).is_hermitian is False
    assert nk.operator.PauliStrings(hi, ["XXIIII"], [1.0]).is_hermitian


def test_operator_algebra_properties():
    """Random real LocalOperators (terms on 1-3 of 4 sites, constants) and random
    even-Y PauliStrings: +, -, scalar *, @ and to_pauli_strings equal the same
    operations on the dense matrices."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    import netket_gb300 as nk
    N = 4
    hi = nk.hilbert.Spin(0.5, N)

    def rand_local(rng, symmetric=False):
        ops, aon = [], []
        for _ in range(int(rng.integers(1, 4))):
            k = int(rng.integers(1, 4))
            sites = sorted(rng.choice(N, size=k, replace=False).tolist())
            m = rng.normal(size=(2 ** k, 2 ** k))
            ops.append(m + m.T if symmetric or rng.random() < 0.5 else m)
            aon.append(sites)
        return nk.operator.LocalOperator(hi, ops, aon, constant=float(rng.normal()))

    def dense(op):
        return _dense_from_local(N, list(op._terms.items()), op.constant)

    # constants within np.isclose(., 0) of zero are dropped by the PauliStrings
    # reduction (base.py:564-576), checked separately below
    @hyp.settings(max_examples=40, deadline=None, derandomize=True, database=None)
    @hyp.given(seed=st.integers(0, 2 ** 31 - 1),
               c=st.floats(-3, 3).filter(lambda v: v == 0 or abs(v) > 1e-6))
    def check(seed, c):
        rng = np.random.default_rng(seed)
        A, B = rand_local(rng), rand_local(rng)
        np.testing.assert_allclose(dense(A + B), dense(A) + dense(B), atol=1e-12)
        np.testing.assert_allclose(dense(A - c * B), dense(A) - c * dense(B), atol=1e-12)
        np.testing.assert_allclose(dense(A @ B), dense(A) @ dense(B), atol=1e-10)
        S = rand_local(rng, symmetric=True)
        assert S.is_hermitian
        P = S.to_pauli_strings()
        np.testing.assert_allclose(_dense_from_pauli(N, P.operators, P.weights).real,
                                   dense(S), atol=1e-10)
        strings = ["".join(rng.choice(list("IXZ"), size=N)) for _ in range(5)]
        w = rng.normal(size=5)
        P1 = nk.operator.PauliStrings(hi, strings[:3], w[:3])
        P2 = nk.operator.PauliStrings(hi, strings[3:], w[3:])
        D = 2.0 * P1 - P2 + c
        ref = 2.0 * _dense_from_pauli(N, strings[:3], w[:3]) - \
            _dense_from_pauli(N, strings[3:], w[3:]) + c * np.eye(2 ** N)
        np.testing.assert_allclose(_dense_from_pauli(N, D.operators, D.weights), ref, atol=1e-10)

    check()
    P = nk.operator.PauliStrings(hi, ["XXII", "IZZI"], [1.0, -0.5])
    T = P + 1e-10
    assert list(T.operators) == list(P.operators) and np.array_equal(T.weights, P.weights)
    assert "IIII" in list((P + 1e-6).operators)


def test_spin_basis_enumeration():
    """Spin._all_local_indices lists every basis state, first site most
    significant, filtered to the fixed number of down spins under total_sz."""
    import itertools
    from netket_gb300.hilbert import Spin
    for N in range(1, 11):
        for tsz in [None] + ([0, 1] if N % 2 == 0 else [0.5, -1.5]):
            if tsz is not None and abs(2 * tsz) > N:
                continue
            h = Spin(0.5, N, total_sz=tsz)
            ref = np.array(list(itertools.product([0, 1], repeat=N)), dtype=np.int8)
            if h.n_down is not None:
                ref = ref[ref.sum(axis=1) == h.n_down]
            got = h._all_local_indices()
            assert got.dtype == np.int8 and np.array_equal(got, ref)
            assert len(got) == h.n_states
    assert Spin(0.5, 4, total_sz=0) == Spin(0.5, 4, total_sz=0)
    assert len({Spin(0.5, 4), Spin(0.5, 4), Spin(0.5, 4, total_sz=0)}) == 2


def test_batched_work_lists():
    """Every instance's chains and samples appear in exactly one work item, in
    blocks of the tuned size, largest instances (N * M) first, with the same
    pairs as a direct enumeration."""
    from netket_gb300.batched import _work_lists, tfim_instances
    inst = tfim_instances(64, seed=5)
    Ns = [N for N, _ in inst]
    Ms = [2 * N for N in Ns]
    for B, L, cpi, spi in [(1024, 4, 4, 8), (16, 3, 8, 5), (7, 1, 2, 3)]:
        cw, ew = _work_lists(Ns, Ms, B, B * L, cpi, spi)
        assert cw.dtype == np.int32 and ew.dtype == np.int32
        cw, ew = cw.reshape(-1, 2), ew.reshape(-1, 2)
        order = sorted(range(len(Ns)), key=lambda i: -Ns[i] * Ms[i])
        ref_c = [(i, b) for i in order for b in range(0, B, cpi)]
        ref_e = [(i, s) for i in order for s in range(0, B * L, spi)]
        assert [tuple(r) for r in cw] == ref_c and [tuple(r) for r in ew] == ref_e
        sizes = [Ns[i] * Ms[i] for i in cw[:, 0]]
        assert sizes == sorted(sizes, reverse=True)
        for i in range(len(Ns)):
            firsts = cw[cw[:, 0] == i, 1]
            covered = np.concatenate([np.arange(f, min(f + cpi, B)) for f in firsts])
            assert np.array_equal(np.sort(covered), np.arange(B))


def test_autotune_cache(tmp_path):
    """The cache keeps other signatures' entries, is replaced atomically, and an
    entry missing a launch parameter (or a corrupt file) is tuned again."""
    from netket_gb300.batched import _cached_launch, _load_tune_cache, _store_tune_choice
    path = str(tmp_path / "sub" / "tune.json")
    assert _load_tune_cache(path) == {}
    good = {"chains_per_item": 4, "sampler_ctas": 1216, "samples_per_item": 8,
            "eloc_ctas": 1216, "tuned_ms": 1.5}
    _store_tune_choice(path, "a", good)
    _store_tune_choice(path, "b", dict(good, chains_per_item=8))
    cache = _load_tune_cache(path)
    assert set(cache) == {"a", "b"} and _cached_launch(cache, "a") == good
    assert _cached_launch(cache, "b")["chains_per_item"] == 8
    assert _cached_launch(cache, "c") is None
    assert not [p for p in os.listdir(tmp_path / "sub") if p.endswith(".tmp")]
    stale = dict(good)
    del stale["eloc_ctas"]
    assert _cached_launch({"a": stale}, "a") is None
    assert _cached_launch({"a": dict(good, sampler_ctas=0)}, "a") is None
    assert _cached_launch({"a": dict(good, sampler_ctas=2.5)}, "a") is None
    assert _cached_launch({"a": "x"}, "a") is None
    with open(path, "w") as f:
        f.write("{not json")
    assert _load_tune_cache(path) == {}
    _store_tune_choice(path, "a", good)
    assert _load_tune_cache(path) == {"a": good}
    with open(path, "w") as f:
        f.write("[1, 2]")
    assert _load_tune_cache(path) == {}


def test_mcstate_sample_count_setters():
    """n_samples / chain_length / n_discard_per_chain / sampler setters follow
    state.py:374-468 (rounding up with a warning, validation, n_samples kept
    across a sampler change, fresh chains from a derived seed)."""
    import warnings
    import torch
    from netket_gb300 import vqs

    class FakeSampler:
        def __init__(self, n_chains):
            self.n_chains = n_chains
            self.seeds = []

        def init_state(self, model, params, seed):
            self.seeds.append(seed)
            return ("state", seed)

    vs = vqs.MCState.__new__(vqs.MCState)
    vs._samples = vs._cache = None
    vs.compute_dtype = torch.float64
    vs._flat = torch.zeros(3, dtype=torch.float64)
    vs.model = None
    vs._sampler_seed = 7
    vs.sampler = FakeSampler(16)
    vs.chain_length = 4
    vs.n_discard_per_chain = None
    assert vs.n_samples == 64 and vs.n_discard_per_chain == 5
    vs._samples = "old"
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        vs.n_samples = 160
    assert vs.chain_length == 10 and vs._samples is None
    with pytest.warns(UserWarning, match="increased to 176"):
        vs.n_samples = 161
    assert vs.n_samples == 176 and vs.n_samples_per_rank == 176
    for bad in (0, -3):
        with pytest.raises(ValueError):
            vs.chain_length = bad
        with pytest.raises(ValueError):
            vs.n_samples = bad
    with pytest.raises(ValueError):
        vs.n_discard_per_chain = -1
    vs.n_discard_per_chain = 0
    assert vs.n_discard_per_chain == 0
    new = FakeSampler(48)
    with pytest.warns(UserWarning):
        vs.sampler = new          # 176 samples -> 4 chains of 48 = 192
    assert vs.sampler is new and vs.n_samples == 192 and vs.chain_length == 4
    assert vs.sampler_state == ("state", new.seeds[0]) and new.seeds[0] != 7
    s1 = vs._sampler_seed
    vs.sampler = FakeSampler(48)
    assert vs._sampler_seed not in (7, s1) and vs.n_samples == 192
    assert vqs._derive_seed(7) == vqs._derive_seed(7) < 2 ** 64


def test_log_psi_to_array():
    import torch
    from netket_gb300.vqs import log_psi_to_array
    rng = np.random.default_rng(2)
    lp = rng.normal(size=64) * 30 + 500.0          # exp overflows without the shift
    psi = log_psi_to_array(torch.as_tensor(lp)).numpy()
    ref = np.exp(lp - lp.max())
    np.testing.assert_allclose(psi, ref / np.linalg.norm(ref), rtol=1e-13)
    assert abs(np.linalg.norm(psi) - 1.0) < 1e-14
    raw = log_psi_to_array(torch.as_tensor(lp[:4] - 500.0), normalize=False).numpy()
    np.testing.assert_allclose(raw, np.exp(lp[:4] - 500.0), rtol=1e-14)
    assert log_psi_to_array(torch.zeros(3, dtype=torch.float32)).dtype == torch.float64


def test_sampler_constructor_checks():
    """metropolis.py:273-325 and base.py:139-154, before any device work."""
    import netket_gb300 as nk
    hi = nk.hilbert.Spin(0.5, 8)
    s = nk.sampler.MetropolisLocal(hi)
    assert s.n_chains == 16 and s.n_chains_per_rank == 16 and s.sweep_size == 8
    assert s.machine_pow == 2 and s.chunk_size is None and not s.is_exact
    assert nk.sampler.MetropolisLocal(hi, n_chains_per_rank=32).n_chains == 32
    assert nk.sampler.MetropolisLocal(hi, n_chains=64, chunk_size=16).chunk_size == 16
    assert nk.sampler.MetropolisLocal(hi, n_chains=8, chunk_size=16).n_chains == 8
    with pytest.raises(ValueError, match="Cannot specify both"):
        nk.sampler.MetropolisLocal(hi, n_chains=16, n_chains_per_rank=16)
    with pytest.raises(ValueError, match="Chunk size must divide"):
        nk.sampler.MetropolisLocal(hi, n_chains=48, chunk_size=32)
    with pytest.raises(TypeError, match="reset_chains"):
        nk.sampler.MetropolisLocal(hi, reset_chains=1)
    with pytest.raises(ValueError, match="must be real"):
        nk.sampler.MetropolisLocal(hi, machine_pow=2j)
    with pytest.raises(ValueError, match="must be positive"):
        nk.sampler.MetropolisLocal(hi, machine_pow=-1)
    with pytest.raises(NotImplementedError, match="machine_pow"):
        nk.sampler.MetropolisLocal(hi, machine_pow=1)
    with pytest.raises(TypeError, match="MetropolisRule"):
        nk.sampler.MetropolisSampler(hi, "local")


def test_pauli_strings_product_golden(golden):
    """PauliStrings @ PauliStrings against the reference's own _matmul
    (pauli_products.npz, made by tests/golden/make_golden.py): strings and
    weights equal where the reduced product is real (imaginary cross terms that
    cancel included), refused where a weight stays imaginary; and the product's
    matrix is the product of the matrices."""
    import netket_gb300 as nk
    g = golden("pauli_products")
    names = sorted({k.split("__")[0] for k in g})
    N = len(str(g[names[0] + "__a_ops"][0]))
    hi = nk.hilbert.Spin(0.5, N)
    n_real = n_refused = 0
    for name in names:
        A = nk.operator.PauliStrings(hi, list(g[name + "__a_ops"]), g[name + "__a_w"])
        B = nk.operator.PauliStrings(hi, list(g[name + "__b_ops"]), g[name + "__b_w"])
        w_ref = g[name + "__weights"]
        if np.any(np.imag(w_ref) != 0):
            with pytest.raises(TypeError, match="complex"):
                A @ B
            n_refused += 1
            continue
        C = A @ B
        assert C.operators == [str(o) for o in g[name + "__ops"]], name
        np.testing.assert_array_equal(np.asarray(C.weights), np.real(w_ref), err_msg=name)
        dA = _dense_from_pauli(N, A.operators, A.weights)
        dB = _dense_from_pauli(N, B.operators, B.weights)
        np.testing.assert_allclose(_dense_from_pauli(N, C.operators, C.weights), dA @ dB,
                                   atol=1e-12, err_msg=name)
        n_real += 1
    assert n_real >= 10 and n_refused >= 5
    P = nk.operator.PauliStrings(hi, ["XX" + "I" * (N - 2), "ZZ" + "I" * (N - 2)], [1.0, 0.5])
    np.testing.assert_allclose(_dense_from_pauli(N, (P ** 3).operators, (P ** 3).weights),
                               np.linalg.matrix_power(_dense_from_pauli(N, P.operators,
                                                                        P.weights), 3),
                               atol=1e-12)
    with pytest.raises(TypeError, match="@"):
        P * P
    with pytest.raises(NotImplementedError):
        P ** 0
    with pytest.raises(ValueError, match="identical hilbert"):
        P @ nk.operator.PauliStrings(nk.hilbert.Spin(0.5, N + 1), "I" * (N + 1))


def test_local_operator_rsub_div_transpose_adjoint():
    """LocalOperator: scalar - op, op / scalar, transpose / T, conjugate, H
    (_local_operator/base.py:263-340, _abstract_operator.py:56-64), adding an
    operator on another Hilbert space fails, the sum keeps the smaller
    mel_cutoff, and ** is repeated @."""
    import netket_gb300 as nk
    N = 3
    hi = nk.hilbert.Spin(0.5, N)
    rng = np.random.default_rng(8)
    m = rng.normal(size=(4, 4))
    A = nk.operator.LocalOperator(hi, [m], [[0, 2]], constant=0.5)
    dA = _dense_from_local(N, list(A._terms.items()), A.constant)

    def dense(op):
        return _dense_from_local(N, list(op._terms.items()), op.constant)

    np.testing.assert_allclose(dense(2.0 - A), 2.0 * np.eye(8) - dA, atol=1e-13)
    np.testing.assert_allclose(dense(A / 4), dA / 4, atol=1e-13)
    np.testing.assert_allclose(dense(A.transpose()), dA.T, atol=1e-13)
    np.testing.assert_allclose(dense(A.T), dA.T, atol=1e-13)
    np.testing.assert_allclose(dense(A.conjugate()), dA, atol=1e-13)
    assert not A.is_hermitian
    np.testing.assert_allclose(dense(A.H), dA.T, atol=1e-13)
    S = A + A.T
    assert S.is_hermitian and S.H is S
    np.testing.assert_allclose(dense(A ** 3), np.linalg.matrix_power(dA, 3), atol=1e-10)
    with pytest.raises(ValueError, match="Dividing by 0"):
        A / 0
    with pytest.raises(TypeError, match="scalar"):
        A / A
    other = nk.operator.LocalOperator(nk.hilbert.Spin(0.5, N + 1), [m], [[0, 1]])
    with pytest.raises(TypeError):
        A + other
    B = nk.operator.LocalOperator(hi, [m], [[1, 2]], mel_cutoff=1e-6)
    assert (A + B).mel_cutoff == min(A.mel_cutoff, 1e-6)


def test_general_lattices_golden(golden):
    """Lattice with basis vectors / site offsets, Triangular, Honeycomb, Kagome:
    edges (order and colours) and site positions equal the reference's own
    get_nn_edges / create_site_positions (lattice_edges.npz, made by
    tests/golden/make_golden.py), hypercubic cases included."""
    import warnings
    import netket_gb300 as nk
    g = golden("lattice_edges")
    names = sorted({k.split("__")[0] for k in g})
    for name in names:
        offs = g[name + "__offsets"]
        lat = nk.graph.Lattice(g[name + "__basis"], list(g[name + "__extent"]),
                               pbc=[bool(b) for b in g[name + "__pbc"]],
                               site_offsets=None if not np.any(offs) and len(offs) == 1 else offs,
                               max_neighbor_order=int(g[name + "__order"]))
        got = np.array(lat.edges(return_color=True), dtype=np.int64).reshape(-1, 3)
        np.testing.assert_array_equal(got, g[name + "__edges"], err_msg=name)
        np.testing.assert_allclose(lat.positions, g[name + "__positions"], atol=1e-12,
                                   err_msg=name)
        assert lat.n_nodes == len(g[name + "__positions"])
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        t = nk.graph.Triangular([4, 3], max_neighbor_order=2)
    np.testing.assert_array_equal(np.array(t.edges(return_color=True)),
                                  g["triangular4x3_nnn__edges"])
    h = nk.graph.Honeycomb([4, 4], max_neighbor_order=3)
    np.testing.assert_array_equal(np.array(h.edges(return_color=True)),
                                  g["honeycomb4_3rd__edges"])
    k = nk.graph.Kagome([3, 3])
    np.testing.assert_array_equal(np.array(k.edges(return_color=True)), g["kagome3__edges"])
    assert h.n_nodes == 32 and k.n_nodes == 27
    with pytest.warns(UserWarning, match="only 2 cells"):
        nk.graph.Triangular([2, 3])
    with pytest.raises(ValueError, match="pbc"):
        nk.graph.Lattice(np.eye(2), [3, 3], pbc=[True])
    with pytest.raises(ValueError, match="extent"):
        nk.graph.Lattice(np.eye(2), [3, 3, 3])
    # a Heisenberg model on the triangular lattice is an ordinary LocalOperator
    hi = nk.hilbert.Spin(0.5, t.n_nodes)
    H = nk.operator.Heisenberg(hi, t, J=[1.0, 0.3])
    assert H.max_conn_size == 1 + t.n_edges


def test_graph_operator_subspace_and_sign_rule_checks():
    """acting_on_subspace (_graph_operator.py:29-44): node i of a smaller graph
    acts on site map[i]; the J-list sign rule is checked per colour subgraph
    (_heisenberg.py:86-100); complex dtypes are refused."""
    import netket_gb300 as nk
    hi = nk.hilbert.Spin(0.5, 6)
    g = nk.graph.Chain(3, pbc=False)
    H = nk.operator.Heisenberg(hi, g, acting_on_subspace=2)
    assert list(H._terms) == [(2, 3), (3, 4)]
    H2 = nk.operator.Heisenberg(hi, g, acting_on_subspace=[5, 0, 3])
    assert list(H2._terms) == [(0, 5), (0, 3)]
    sx = np.array([[0.0, 1.0], [1.0, 0.0]])
    G = nk.operator.GraphOperator(hi, g, site_ops=[sx], acting_on_subspace=[1, 4, 5])
    assert sorted(G._terms) == [(1,), (4,), (5,)]
    with pytest.raises(ValueError, match="length graph.n_nodes"):
        nk.operator.Heisenberg(hi, g, acting_on_subspace=[0, 1])
    with pytest.raises(TypeError, match="list or single integer"):
        nk.operator.Heisenberg(hi, g, acting_on_subspace=(0, 1, 2))
    with pytest.raises(TypeError, match="complex"):
        nk.operator.Heisenberg(hi, g, dtype=np.complex128)
    # J list with nn + nnn colours: on an even periodic square lattice both
    # colour subgraphs are bipartite (x mod 2 colours the nnn bonds too), on an
    # odd one neither is
    hs = nk.hilbert.Spin(0.5, 16)
    sq4 = nk.graph.Square(4, max_neighbor_order=2)
    nk.operator.Heisenberg(hs, sq4, J=[1.0, 0.5], sign_rule=[True, True])
    sq5 = nk.graph.Square(5, max_neighbor_order=2)
    h5 = nk.hilbert.Spin(0.5, 25)
    nk.operator.Heisenberg(h5, sq5, J=[1.0, 0.5], sign_rule=[False, False])
    with pytest.raises(ValueError, match="non-bipartite"):
        nk.operator.Heisenberg(h5, sq5, J=[1.0, 0.5], sign_rule=[False, True])
    with pytest.raises(ValueError, match="one sign_rule entry"):
        nk.operator.Heisenberg(hs, sq4, J=[1.0, 0.5], sign_rule=[True])
    tri = nk.graph.Triangular([3, 3])
    with pytest.raises(ValueError, match="non-bipartite"):
        nk.operator.Heisenberg(nk.hilbert.Spin(0.5, 9), tri, sign_rule=True)
    assert not tri.is_bipartite()


def test_exact_diagonalisation_wrappers():
    """lanczos_ed (with and without matrix_free, with eigenvectors) and full_ed on
    an operator whose matrix is a CPU TFIM from the oracle."""
    import scipy.sparse as sp
    from netket_gb300 import exact
    from oracle import exact as oex
    from oracle import operator as oop
    N = 8
    edges = np.array([(i, (i + 1) % N) for i in range(N)])

    class CpuOp:
        def to_sparse(self):
            x = 1 - 2 * ((np.arange(2 ** N)[:, None] >> np.arange(N - 1, -1, -1)) & 1)
            return sp.csr_matrix(oex.to_sparse_from_conn(
                lambda s: oop.ising_get_conn_padded(s, edges, 1.0, 1.0), x.astype(np.int8)))

        def to_dense(self):
            return self.to_sparse().toarray()

    op = CpuOp()
    ref = np.linalg.eigvalsh(op.to_dense())
    np.testing.assert_allclose(exact.lanczos_ed(op, k=3), ref[:3], rtol=1e-10)
    np.testing.assert_allclose(exact.lanczos_ed(op, k=2, matrix_free=True), ref[:2], rtol=1e-10)
    w, v = exact.lanczos_ed(op, k=2, compute_eigenvectors=True)
    np.testing.assert_allclose(w, ref[:2], rtol=1e-10)
    np.testing.assert_allclose(op.to_dense() @ v, v * w, atol=1e-8)
    np.testing.assert_allclose(exact.full_ed(op), ref, rtol=1e-12, atol=1e-12)
    w2, v2 = exact.full_ed(op, compute_eigenvectors=True)
    np.testing.assert_allclose(w2, ref, rtol=1e-12, atol=1e-12)
    # the example in the reference's lanczos_ed docstring (8-site Ising, h = 1)
    np.testing.assert_allclose(exact.lanczos_ed(op, k=3), [-10.25166179, -10.05467898,
                                                          -8.69093921], atol=1e-8)
    assert abs(ref[0] - oex.tfim_ground_energy(N, 1.0, 1.0)) < 1e-9


def test_stats_printing_and_aliases(golden):
    """Stats prints as the reference's _format_main_string (stats_format.npz,
    made by tests/golden/make_golden.py) and answers to its alias names."""
    from netket_gb300.stats import Stats, _format_mean_error
    g = golden("stats_format")
    for v, s in zip(g["values"], g["strings"]):
        assert _format_mean_error(*v) == str(s)
    st = Stats(-1.5, 0.02, 0.3, 1.5, 1.01)
    assert repr(st) == _format_mean_error(-1.5, 0.02, 0.3) + ", R̂=1.010]"
    assert repr(Stats(1.0, 0.1, 0.2)) == _format_mean_error(1.0, 0.1, 0.2) + "]"
    assert (st.Mean, st.Sigma, st.Variance, st.R, st.TauCorr) == (-1.5, 0.02, 0.3, 1.01, 1.5)
    assert np.isnan(st.tau_corr_max) and np.isnan(st.TauCorrMax) and st.shape == ()
    assert st.replace(mean=2.0).mean == 2.0 and st.replace(mean=2.0).Sigma == 0.02
    assert st.real().mean == -1.5 and st.imag().mean == 0.0
    with pytest.raises(AttributeError):
        st.nothing


def test_sr_qgt_selection():
    """SR picks the QGT form as QGTAuto does for an RBM (qgt/default.py:58-97):
    on the fly with CG unless a dense solver is given; explicit forms win."""
    import netket_gb300 as nk
    o = nk.optimizer
    assert (o.SR().qgt, o.SR().solver) == ("onthefly", "cg")
    assert o.SR(diag_shift=0.1).diag_shift == 0.1
    assert o.SR(solver=o.solver.cholesky_with_fallback).qgt == "dense"
    assert o.SR(o.qgt.QGTAuto, "cholesky").qgt == "dense"
    assert o.SR(o.qgt.QGTJacobianDense).qgt == "dense"
    assert o.SR(qgt=o.qgt.QGTJacobianDense()).solver == "cholesky"
    assert o.SR(o.qgt.QGTOnTheFly, solver_restart=True).solver_restart
    assert o.SR(qgt="dense").qgt == "dense" and o.SR(qgt="onthefly").qgt == "onthefly"
    with pytest.raises(ValueError, match="dense solver"):
        o.SR(o.qgt.QGTOnTheFly, o.solver.cholesky_with_fallback)
    with pytest.raises(ValueError, match="qgt must be"):
        o.SR(qgt="sparse")
    with pytest.raises(NotImplementedError, match="diag_scale"):
        o.SR(diag_scale=0.01)
    with pytest.raises(NotImplementedError, match="holomorphic"):
        o.SR(holomorphic=True)
    with pytest.raises(NotImplementedError, match="linear_solver"):
        o.SR(solver=o.solver.pinv_smooth)
    with pytest.raises(NotImplementedError, match="not supported"):
        o.SR(solver=lambda A, b: b)


def test_rbm_param_dtype_spellings():
    """param_dtype as NetKet scripts write it selects the same precision
    (float / np.float64 / "float64" -> FP64; np.float32 -> FP32); complex and
    JAX-only arguments are refused before any device work."""
    import torch
    import netket_gb300 as nk
    for dt in (float, np.float64, "float64", torch.float64, np.dtype("float64")):
        assert nk.models.RBM(param_dtype=dt).param_dtype == torch.float64
    for dt in (np.float32, "float32", torch.float32):
        assert nk.models.RBM(param_dtype=dt).param_dtype == torch.float32
    for dt in (complex, np.complex128, torch.complex64):
        with pytest.raises(NotImplementedError):
            nk.models.RBM(param_dtype=dt)
    with pytest.raises(NotImplementedError):
        nk.models.RBM(param_dtype=np.int32)
    with pytest.raises(ValueError):
        nk.models.RBM(param_dtype=object())
    with pytest.raises(NotImplementedError, match="initialiser"):
        nk.models.RBM(kernel_init=lambda *a: None)
    with pytest.raises(NotImplementedError, match="activation"):
        nk.models.RBM(activation=np.tanh)

    def log_cosh(x):
        return x
    assert nk.models.RBM(activation=log_cosh).alpha == 1
    with pytest.raises(NotImplementedError, match="precision"):
        nk.models.RBM(precision="highest")
    with pytest.raises(ValueError, match="alpha"):
        nk.models.RBM(alpha=0)


def test_spin_space_products_and_arguments():
    """Spin(s=1/2)**8 and Spin * Spin as in spin.py:201-207; constrained
    products, custom constraints and the inverted ordering are refused."""
    from netket_gb300.hilbert import Spin
    assert Spin(s=1 / 2) ** 8 == Spin(0.5, 8)
    assert Spin(0.5, 3) * Spin(0.5, 5) == Spin(0.5, 8)
    assert Spin(0.5, 4, inverted_ordering=False).N == 4
    for bad in (lambda: Spin(0.5, 4, total_sz=0) ** 2,
                lambda: Spin(0.5, 4, total_sz=0) * Spin(0.5, 2),
                lambda: Spin(0.5, 4, inverted_ordering=True),
                lambda: Spin(0.5, 4, constraint=object()),
                lambda: Spin(1.0, 4)):
        with pytest.raises(NotImplementedError):
            bad()
    with pytest.raises(ValueError):
        Spin(0.5, 0)
    with pytest.raises(TypeError):
        Spin(0.5, 2) ** 0.5


def test_expect_and_grad_formula_choice_refusals():
    """expect_and_grad picks the covariance formula by use_covariance (default:
    the operator's is_hermitian, expect_grad.py:42-64); the non-hermitian
    formula and mutable collections are refused before any device work."""
    import netket_gb300 as nk
    from netket_gb300 import vqs
    hi = nk.hilbert.Spin(0.5, 4)
    vs = vqs.MCState.__new__(vqs.MCState)
    sp = nk.operator.spin
    with pytest.raises(NotImplementedError, match="use_covariance=False"):
        vs.expect_and_grad(sp.sigmap(hi, 1))
    with pytest.raises(NotImplementedError, match="use_covariance=False"):
        vs.expect_and_grad(sp.sigmax(hi, 1), use_covariance=False)
    with pytest.raises(NotImplementedError, match="mutable"):
        vs.expect_and_grad(sp.sigmax(hi, 1), mutable=True)
    with pytest.raises(NotImplementedError, match="mutable"):
        vs.expect_and_forces(sp.sigmax(hi, 1), mutable="batch_stats")


def test_ising_algebra():
    """Ising combined with scalars and LocalOperators equals the dense-matrix
    algebra (NetKet sums lazily; here the sum is a concrete LocalOperator), a
    scalar multiple stays an Ising with h and J scaled."""
    import netket_gb300 as nk
    N = 4
    hi = nk.hilbert.Spin(0.5, N)
    I = nk.operator.Ising(hi, nk.graph.Chain(N), h=0.7, J=1.3)
    Z0 = nk.operator.spin.sigmaz(hi, 0)
    X2 = nk.operator.spin.sigmax(hi, 2)

    def dense(op):
        op = op.to_local_operator() if isinstance(op, nk.operator.Ising) else op
        return _dense_from_local(N, list(op._terms.items()), op.constant)

    dI, dZ, dX = dense(I), dense(Z0), dense(X2)
    two = 2 * I
    assert isinstance(two, nk.operator.Ising) and (two.h, two.J) == (1.4, 2.6)
    np.testing.assert_allclose(dense(-I), -dI, atol=1e-13)
    np.testing.assert_allclose(dense(I / 2), dI / 2, atol=1e-13)
    np.testing.assert_allclose(dense(I + 0.5 * Z0), dI + 0.5 * dZ, atol=1e-13)
    np.testing.assert_allclose(dense(Z0 + I), dZ + dI, atol=1e-13)
    np.testing.assert_allclose(dense(1.5 - I), 1.5 * np.eye(2 ** N) - dI, atol=1e-13)
    np.testing.assert_allclose(dense(I - X2), dI - dX, atol=1e-13)
    np.testing.assert_allclose(dense(I + I), 2 * dI, atol=1e-13)
    np.testing.assert_allclose(dense(I @ Z0), dI @ dZ, atol=1e-12)
    np.testing.assert_allclose(dense(Z0 @ I), dZ @ dI, atol=1e-12)
    np.testing.assert_allclose(dense(I ** 2), dI @ dI, atol=1e-12)
    assert (I + Z0).is_hermitian and I.is_hermitian
    with pytest.raises(TypeError, match="complex"):
        nk.operator.Ising(hi, nk.graph.Chain(N), h=1.0, dtype=np.complex64)
    with pytest.raises(TypeError, match="complex"):
        I * 1j


def test_sampler_state_counters():
    """acceptance / n_steps / n_accepted as the reference's MetropolisSamplerState
    (metropolis.py:96-130): None before any step since the last reset."""
    import torch
    from netket_gb300.sampler import MetropolisSamplerState
    st = MetropolisSamplerState(torch.zeros((4, 3), dtype=torch.int8),
                                torch.zeros(4, dtype=torch.float64), 7, 0,
                                torch.zeros(4, dtype=torch.int64))
    assert st.acceptance is None and st.n_steps == 0 and "accepted" not in repr(st)
    st.n_accepted_proc = torch.tensor([3, 1, 0, 2])
    st.n_steps_proc = 24
    assert st.n_accepted == 6 and st.n_steps == 24 and st.acceptance == 0.25
    assert "# accepted = 6/24 (25.0%)" in repr(st)


def test_nn_log_cosh(golden):
    """nk.nn.log_cosh equals the reference's log_cosh (logcosh.npz) and is the
    activation the RBM accepts."""
    import torch
    import netket_gb300 as nk
    g = golden("logcosh")
    np.testing.assert_allclose(nk.nn.log_cosh(g["x"]), g["y"], rtol=1e-14, atol=1e-15)
    t = nk.nn.log_cosh(torch.as_tensor(g["x"]))
    np.testing.assert_allclose(t.numpy(), g["y"], rtol=1e-14, atol=1e-15)
    assert nk.models.RBM(alpha=2, activation=nk.nn.log_cosh).alpha == 2


def test_local_operator_refuses_imaginary_elements():
    """A complex term (sigma^y) or complex constant raises instead of losing its
    imaginary part; complex-typed matrices with zero imaginary part are kept."""
    import warnings
    import netket_gb300 as nk
    hi = nk.hilbert.Spin(0.5, 2)
    sy = np.array([[0, -1j], [1j, 0]])
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        with pytest.raises(TypeError, match="complex"):
            nk.operator.LocalOperator(hi, [sy], [[0]])
        with pytest.raises(TypeError, match="complex"):
            nk.operator.LocalOperator(hi, constant=1j)
        with pytest.raises(TypeError, match="complex"):
            nk.operator.LocalOperator(hi, dtype=np.complex128)
        op = nk.operator.LocalOperator(hi, [np.array([[0, 1], [1, 0]], dtype=complex)], [[1]],
                                       constant=2 + 0j)
    assert op.constant == 2.0 and op._terms[(1,)].dtype == np.float64
    np.testing.assert_array_equal(op._terms[(1,)], [[0.0, 1.0], [1.0, 0.0]])


def test_parameter_assignment_forms():
    """vs.parameters accepts a pytree of NumPy arrays (as loaded from a file) and
    tensors; complex values and a wrong size are refused, not cast."""
    import torch
    from netket_gb300 import vqs
    from netket_gb300.models import RBM
    vs = vqs.MCState.__new__(vqs.MCState)
    vs.model = RBM(alpha=1)
    vs.N, vs.M = 2, 2
    vs._flat = torch.zeros(8, dtype=torch.float64)
    vs._version, vs._samples, vs._cache = 0, None, None
    p = {"Dense": {"bias": np.array([1.0, 2.0]), "kernel": np.arange(4.0).reshape(2, 2)},
         "visible_bias": [7.0, 8.0]}
    vs.parameters = p
    np.testing.assert_array_equal(vs._flat.numpy(), [1, 2, 0, 1, 2, 3, 7, 8])
    assert vs._version == 1
    vs.flat_parameters = torch.arange(8, dtype=torch.float32)
    np.testing.assert_array_equal(vs._flat.numpy(), np.arange(8.0))
    with pytest.raises(TypeError, match="complex"):
        vs.flat_parameters = np.ones(8) * (1 + 1j)
    with pytest.raises(TypeError, match="complex"):
        vs.parameters = dict(p, visible_bias=np.array([1j, 0]))
    with pytest.raises(ValueError, match="expected 8"):
        vs.flat_parameters = np.ones(7)


def test_precision_progress_bar_switch():
    """expect_to_precision(verbose=): no bar when False; a tqdm bar (or nothing
    without tqdm) when True."""
    from netket_gb300.vqs import _progress_bar
    assert _progress_bar(False, 10) is None
    bar = _progress_bar(True, 10)
    try:
        import tqdm  # noqa: F401
        assert bar is not None
        bar.update(1)
        bar.close()
    except ImportError:
        assert bar is None

"""Benchmark: VMC steps/s of the 10x10 J1-J2 Heisenberg minSR step on one GB300.

Workload (the configuration the metric is quoted on): 10x10 periodic square
lattice, J1 = 1, J2 = 0.5, total Sz = 0; RBM alpha = 4 (M = 400, P = 40,500);
MetropolisExchange on the 400 nearest and next-nearest bonds, 4096 chains,
16,384 samples per step (4 per chain), 5 discarded sweeps per chain; minSR with
T = O_L O_L^T + 1e-4 I (16,384 x 16,384) solved to an FP64 residual; SGD lr 0.01.
Synthetic: random RBM initialisation (Normal(0, 0.01)), no dataset.

A step = one VMC_SR step (sample, local energies, statistics, T, solve,
parameter update), through ``netket_gb300.driver.VMC_SR.advance``.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

The line carries: ``roofline`` (the solve, the step's largest phase),
``roofline_gram``, ``matched_energy`` (each arm's energy error against an
all-FP64 run over a few steps on the same samples), ``plain_fp32`` (the plain
FP32 GPU path), ``cpu_baseline`` and ``e2e`` (host buffers through the public
API).  ``--impl reference`` times the reference algorithm on the host cores (the
numpy FP64 restatement in ``oracle/``; NetKet's own JAX path cannot be
installed here): every phase of the full 16,384-sample step is measured, the
per-sample phases on a 1/32 slice of the chains.  Under torchrun every rank
runs an independent replica (the path has no cross-GPU exchange on a
single-GPU machine); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import statistics as pystats
import subprocess
import sys
import time

NPROC = os.cpu_count() or 1
for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ.setdefault(var, str(NPROC))

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {
    "workload": "j1j2_10x10_minsr",
    "lattice": "10x10 periodic square, J1=1, J2=0.5, total_sz=0, sign_rule=[True, False]",
    "model": "RBM alpha=4 (M=400, P=40500)",
    "sampler": "MetropolisExchange nn+nnn bonds (400 clusters)",
    "n_chains": 4096, "n_samples": 16384, "n_discard_per_chain": 5,
    "solver": "minSR, T 16384x16384, diag_shift=1e-4", "lr": 0.01,
}
METRIC = "VMC steps/s"
# the large configuration (``--workload large``): 16x16 Heisenberg, alpha 8,
# 65,536 samples, a 65,536 x 65,536 T
LARGE = {
    "workload": "heisenberg_16x16_alpha8_minsr",
    "lattice": "16x16 periodic square, J=1, total_sz=0, sign_rule=True",
    "model": "RBM alpha=8 (M=2048, P=526592)",
    "sampler": "MetropolisExchange nn bonds (512 clusters)",
    "n_chains": 16384, "n_samples": 65536, "n_discard_per_chain": 5,
    "solver": "minSR, T 65536x65536, diag_shift=1e-4", "lr": 0.005,
}


def workload_config(args, world):
    if args.workload == "large":
        return dict(LARGE, precision=args.precision, parallelism=f"replicas{world}",
                    l2="per-step working set > L2: T64 34.4 GB + T32 17.2 GB")
    cfg = dict(WORKLOAD, precision=args.precision, parallelism=f"replicas{world}",
               l2="per-step working set > L2: T64 2.1 GB + T32 1.1 GB")
    if (args.n_chains, args.n_samples) != (WORKLOAD["n_chains"], WORKLOAD["n_samples"]):
        n = args.n_samples
        cfg.update(workload=f"j1j2_10x10_minsr_n{n}", n_chains=args.n_chains, n_samples=n,
                   solver=f"minSR, T {n}x{n}, diag_shift=1e-4",
                   l2=f"T64 {8 * n * n / 1e9:.2f} GB + T32 {4 * n * n / 1e9:.2f} GB")
    return cfg


def build_large(nk, precision, seed=0):
    """16x16 Heisenberg (J = 1, Marshall sign rule, total Sz = 0), RBM alpha 8,
    MetropolisExchange on the nearest-neighbour bonds, 16,384 chains x 4 samples,
    minSR with diag_shift 1e-4, SGD lr 0.005 (at lr 0.01 this run diverges after
    about ten steps: the energy turns back up and the local energies blow up)."""
    g = nk.graph.Square(16)
    hi = nk.hilbert.Spin(0.5, N=256, total_sz=0)
    H = nk.operator.Heisenberg(hi, g, J=1.0, sign_rule=True)
    sampler = nk.sampler.MetropolisExchange(hi, graph=g, n_chains=LARGE["n_chains"])
    vs = nk.vqs.MCState(sampler, nk.models.RBM(alpha=8), n_samples=LARGE["n_samples"],
                        n_discard_per_chain=5, seed=seed, precision=precision)
    drv = nk.driver.VMC_SR(H, nk.optimizer.Sgd(LARGE["lr"]), diag_shift=1e-4,
                           variational_state=vs, use_ntk=True)
    return H, vs, drv


def build_problem(nk, precision, seed=0, n_chains=4096, n_samples=16384):
    g = nk.graph.Square(10, max_neighbor_order=2)
    hi = nk.hilbert.Spin(0.5, N=100, total_sz=0)
    # Marshall's sign rule on the bipartite J1 bonds (a positive RBM cannot carry
    # the J1 sign structure; with NetKet's default [False, False] the FP64 and
    # the mixed runs both diverge after ~15 steps)
    H = nk.operator.Heisenberg(hi, g, J=[1.0, 0.5], sign_rule=[True, False])
    sampler = nk.sampler.MetropolisExchange(hi, graph=g, d_max=1, n_chains=n_chains)
    vs = nk.vqs.MCState(sampler, nk.models.RBM(alpha=4), n_samples=n_samples,
                        n_discard_per_chain=5, seed=seed, precision=precision)
    drv = nk.driver.VMC_SR(H, nk.optimizer.Sgd(0.01), diag_shift=1e-4, variational_state=vs,
                           use_ntk=True)
    return H, vs, drv


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", f"vmck_clocks_{os.getpid()}.csv")

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        try:
            for line in open(self.path):
                f = [v.strip() for v in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1].split()[0]))
                    mx = float(f[2].split()[0])
                except ValueError:
                    continue
                names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                         "sw_power_cap"]
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        except OSError:
            pass
        return {"sm_mhz": pystats.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(value, dist=None, device="cpu"):
    """The largest value over all ranks (``dist`` is ``torch.distributed`` or
    None): replicas are timed together, so the job takes as long as its slowest
    rank."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, ms_max):
    """Whole-job steps/s of ``world`` replicas whose slowest takes ms_max per step."""
    return world * 1000.0 / ms_max


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _pin_samples(vs):
    """Make ``vs`` take its samples from ``box["x"]`` instead of its own sampler."""
    box = {}
    vs.reset = lambda: None

    def sample(**kw):
        vs._samples = box["x"]
        return vs._samples
    vs.sample = sample
    return box


def matched_energy(nk, steps, n_chains, n_samples, seed):
    """Energy error of each arm against the all-FP64 run over ``steps`` minSR steps
    from the same initial parameters: the mixed path (this library's default) and
    the plain FP32 GPU path (dense connected elements, materialised Jacobian,
    cuBLAS SSYRK, cuSOLVER SPOTRF) take the FP64 run's samples at every step and
    their own parameters, so the energies differ by arithmetic only.  Target:
    within 1e-4 relative of the FP64 run."""
    import torch
    _, v64, d64 = build_problem(nk, "fp64", seed=seed, n_chains=n_chains, n_samples=n_samples)
    arms = {}
    for name, prec in (("mixed", "mixed"), ("fp32_plain", "fp32")):
        _, v, d = build_problem(nk, prec, seed=seed, n_chains=n_chains, n_samples=n_samples)
        if name == "fp32_plain":
            v.local_estimator = "dense"
            d.gram = "dense"
            d.solve = "cholesky"
        v.flat_parameters = v64.flat_parameters.clone()
        arms[name] = (v, d, _pin_samples(v))
    dev = {k: 0.0 for k in arms}
    e64 = []
    t0 = time.perf_counter()
    for _ in range(steps):
        s64, u64 = d64.compute_loss_and_update()
        x = v64.samples.clone()
        d64.update_parameters(u64)
        d64.step_count += 1
        e64.append(s64.mean)
        for name, (v, d, box) in arms.items():
            box["x"] = x
            s, u = d.compute_loss_and_update()
            d.update_parameters(u)
            d.step_count += 1
            dev[name] = max(dev[name], abs(s.mean - s64.mean) / abs(s64.mean))
    torch.cuda.synchronize()
    return {"steps": steps, "target_rel": 1e-4,
            "max_rel_energy_error_vs_fp64": {k: float(f"{v:.3e}") for k, v in dev.items()},
            "within_target": {k: v <= 1e-4 for k, v in dev.items()},
            "fp64_energy_per_site_first_last": [round(e64[0] / 100, 8), round(e64[-1] / 100, 8)],
            "wall_s": round(time.perf_counter() - t0, 1),
            "how": "the mixed and plain FP32 arms run on the FP64 run's samples (same "
                   "initial parameters, own parameters afterwards)"}


def run_ours(args):
    import torch
    import netket_gb300 as nk
    from netket_gb300 import _native
    from netket_gb300.driver import PhaseTimer

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    large = args.workload == "large"
    if large:
        H, vs, drv = build_large(nk, args.precision, seed=rank)
    else:
        H, vs, drv = build_problem(nk, args.precision, seed=rank, n_chains=args.n_chains,
                                   n_samples=args.n_samples)
    drv.advance(args.warmup)
    barrier()
    L = _native.lib()
    launches0 = L.vmck_launch_count()
    drv.phase_timer = PhaseTimer()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        start.record()
        for _ in range(args.steps):
            st = drv.advance(1)
        stop.record()
        barrier()
    launches = L.vmck_launch_count() - launches0
    phases = drv.phase_timer.summary()
    drv.phase_timer = None
    ms = start.elapsed_time(stop) / args.steps
    ms_max = max_over_ranks(ms, dist, "cuda")
    value = replica_throughput(world, ms_max)
    energy = st.mean / vs.N

    # ---------------- end to end through the public API, host buffers
    P = vs.n_parameters
    h_params = torch.empty(P, dtype=torch.float64).pin_memory()
    h_params.copy_(vs.flat_parameters.cpu())
    h_out = torch.empty(P + 5, dtype=torch.float64).pin_memory()
    barrier()
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        vs.flat_parameters.copy_(h_params, non_blocking=True)
        vs.params_changed()
        st = drv.advance(1)
        h_out[:P].copy_(vs.flat_parameters, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        h_out[P:] = torch.tensor([st.mean, st.error_of_mean, st.variance, st.tau_corr, st.R_hat])
        h_params.copy_(h_out[:P])
    e1.record()
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e_value = replica_throughput(world, max_over_ranks(e2e_ms, dist, "cuda"))

    # ---------------- the plain FP32 GPU path (reference algorithm on the GPU)
    plain = None
    if large:
        plain = {"skipped": "the dense FP32 Jacobian of this size (65536 x 526592) is 138 GB"}
    elif args.plain_steps > 0:
        _, vs32, drv32 = build_problem(nk, "fp32", seed=rank, n_chains=args.n_chains,
                                       n_samples=args.n_samples)
        vs32.local_estimator = "dense"
        drv32.gram = "dense"
        drv32.solve = "cholesky"
        drv32.advance(2)
        barrier()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record()
        for _ in range(args.plain_steps):
            st32 = drv32.advance(1)
        p1.record()
        barrier()
        pms = p0.elapsed_time(p1) / args.plain_steps
        plain = {"path": "fp32 dense: get_conn + logpsi on every row, materialised Jacobian, "
                         "cuBLAS SSYRK T, cuSOLVER SPOTRF",
                 "ms_per_step": round(pms, 3), "steps_per_s": round(1000.0 / pms, 4),
                 "speedup_of_value": round(pms / ms_max, 3)}
        del vs32, drv32

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return None
    peaks = load_peaks()
    n = vs.n_samples
    # dominant phase: the solve (FP32 tensor-core Cholesky of T + refinement against
    # the FP64 T), algorithmic work n^3 / 3 flop of the factorisation
    solve_ms = phases.get("solve")
    roof = None
    if solve_ms:
        chol_flops = float(n) ** 3 / 3.0
        achieved = chol_flops / (solve_ms * 1e-3) / 1e12
        if large or args.n_samples != WORKLOAD["n_samples"]:
            args.solve_traffic = None  # measured for the 16,384 case only
        roof = {"kernel": "minSR solve: Cholesky of T (chol_leaf_kernel + tcgen05 tc_gemm_kernel, "
                          "FP16 hi/lo split, 3 products) + iterative refinement (trsv, symv)",
                "bound": "tensor", "achieved": round(achieved, 3), "peak": peaks["bf16_tflops"],
                "unit": "TFLOP/s", "frac": round(achieved / peaks["bf16_tflops"], 5),
                "traffic": args.solve_traffic, "peak_source": peaks["source"],
                "algorithmic_flops_per_launch": chol_flops,
                "executed_tensor_tflops": round(3 * chol_flops / (solve_ms * 1e-3) / 1e12, 3),
                "launch_ms": round(solve_ms, 4),
                "note": "one 'launch' = the solve phase of one step (CUDA events around it); "
                        "executed tensor flops count the three FP16 products per FP32 "
                        "multiply-add of the factorisation; traffic = DRAM bytes of one solve "
                        "from the ncu capture in profiles/"}
    gram_ms = phases.get("gram")
    roof_gram = None
    if gram_ms:
        M = vs.M
        flops = float(n) * (n + 1) * M  # lower triangle of t t^T (n x n x M), 2 flop per FMA
        if M <= nk.ngd.TC_GRAM_MAX_M:
            # hi*hi, hi*lo, lo*hi, lo*lo over K padded to a multiple of 64
            executed = float(n) * (n + 1) * 4 * (-(-M // 64) * 64)
            kname = "structured Gram T = O_L O_L^T (gram_tc_kernel, tcgen05, fused epilogue)"
            traffic = args.gram_traffic if args.gram_traffic is not None else \
                (73.9e6 + 346.2e6) * (n / 8192.0) ** 2
        else:
            # hi*hi, hi*lo, lo*hi, lo*lo over K padded to 64
            executed = float(n) * (n + 1) * 4 * (-(-M // 64) * 64)
            kname = ("structured Gram T = O_L O_L^T (tcgen05 tc_gemm_kernel, FP16 hi/lo, "
                     "drained accumulation, + gram_assemble_kernel)")
            # DRAM bytes of the GEMM and the assembly pass at n = 16,384 (ncu,
            # profiles/j1j2_10x10_minsr_step_launches.md), n^2 for other sizes
            traffic = args.gram_traffic if args.gram_traffic is not None else \
                (0.525e9 + 2.085e9) * (n / 16384.0) ** 2
        achieved = flops / (gram_ms * 1e-3) / 1e12
        roof_gram = {"kernel": kname,
                     "bound": "tensor", "achieved": round(achieved, 3),
                     "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                     "frac": round(achieved / peaks["bf16_tflops"], 5), "traffic": traffic,
                     "algorithmic_flops_per_launch": flops,
                     "executed_tensor_tflops": round(executed / (gram_ms * 1e-3) / 1e12, 3),
                     "launch_ms": round(gram_ms, 4)}
    matched = None
    if large:
        matched = {"skipped": "the all-FP64 arm at this size is measured by --precision fp64"}
    elif args.matched_steps > 0:
        matched = matched_energy(nk, args.matched_steps, args.n_chains, args.n_samples, rank)
    cpu = None
    if not args.no_cpu_baseline and not large:
        cpu = run_cpu_baseline()
    line = {
        "metric": METRIC, "value": round(value, 5), "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else args.precision, "data": "synthetic",
        "config": workload_config(args, world),
        "samples_per_s": round(value * n, 1),
        "energy_per_site": round(energy, 8),
        "phases_ms": {k: round(v, 4) for k, v in phases.items()},
        "plain_fp32": plain,
        "roofline": roof,
        "roofline_gram": roof_gram,
        "matched_energy": matched,
        "cpu_baseline": cpu,
        "e2e": {"value": round(e2e_value, 5), "unit": "steps/s",
                "h2d_bytes_per_step": P * 8, "d2h_bytes_per_step": P * 8 + 6 * 8},
        "gpu_launches": int(launches),
        "gpu_launches_per_step": round(launches / args.steps, 2),
        "clocks": clk.summary(),
    }
    if dist:
        dist.destroy_process_group()
    return line


def run_batched(args):
    """Batched workload: 64 independent 1D TFIM instances (N drawn uniformly from
    {16, 24, ..., 144}, h uniform in [0.5, 1.5], seed 0), RBM alpha = 2 with FP32
    parameters, MetropolisLocal with 1024 chains x 4 samples each, minSR with the
    refined solve.  One step advances all 64 instances: persistent sampler and
    local-energy launches over an (instance, chain block) work queue with
    autotuned launch shapes, the per-instance updates on 8 streams, the whole
    step one CUDA graph.  Each instance's parameters equal its single-instance
    run bit for bit (tests/test_gpu_batched.py).  Compared against the same 64
    instances stepped one after another through MCState + VMC_SR."""
    import torch
    import netket_gb300 as nk
    from netket_gb300 import batched as nb

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    inst = nb.tfim_instances(64, seed=0)
    B, L = 1024, 4
    bt = nb.BatchedTFIM(inst, n_chains=B, chain_length=L, n_discard=5, diag_shift=1e-4,
                        lr=0.01, seed=1000 * rank)
    for _ in range(args.warmup - 1):
        bt.step()
    bt.capture()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        a.record()
        for _ in range(args.steps):
            bt.graph.replay()
        b.record()
        torch.cuda.synchronize()
    ms = a.elapsed_time(b) / args.steps
    ms_max = max_over_ranks(ms)
    # end to end: graph replay + the device-to-host read of every instance's
    # statistics and solver status, per step
    e0 = time.perf_counter()
    for _ in range(args.steps):
        _, status = bt.step()
    e2e_ms = (time.perf_counter() - e0) * 1e3 / args.steps
    bad = int((status != 0).sum())
    # sequential baseline: each instance alone through the public single-problem API
    seq_ms = None
    if rank == 0:
        seq = []
        for i, (N, h) in enumerate(inst):
            hi = nk.hilbert.Spin(0.5, N)
            H = nk.operator.Ising(hi, nk.graph.Chain(N), h=h)
            vs = nk.vqs.MCState(nk.sampler.MetropolisLocal(hi, n_chains=B),
                                nk.models.RBM(alpha=2, param_dtype=torch.float32),
                                n_samples=B * L, n_discard_per_chain=5, seed=i,
                                sampler_seed=i + 1, precision="mixed")
            drv = nk.driver.VMC_SR(H, nk.optimizer.Sgd(0.01), diag_shift=1e-4,
                                   variational_state=vs, use_ntk=True, gram_mode=1,
                                   solve="refined")
            drv.advance(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            drv.advance(2)
            torch.cuda.synchronize()
            seq.append((time.perf_counter() - t0) * 1e3 / 2)
            del vs, drv
        seq_ms = sum(seq)
    if rank != 0:
        return None
    Ns = sorted(N for N, _ in inst)
    return {
        "metric": "batched VMC steps/s (64 TFIM instances per step)",
        "value": round(replica_throughput(world, ms_max), 4), "unit": "steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_max, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "batched_tfim_64", "instances": 64,
                   "N": f"{Ns[0]}..{Ns[-1]} (seeded uniform over 16, 24, ..., 144)",
                   "h": "uniform [0.5, 1.5], seed 0", "model": "RBM alpha=2 FP32",
                   "n_chains": B, "samples_per_instance": B * L,
                   "solver": "minSR per instance, refined FP64 solve",
                   "parallelism": f"replicas{world}", "launch": bt.launch},
        "instance_steps_per_s": round(64 * replica_throughput(world, ms_max), 2),
        "sequential": {"ms_per_step": round(seq_ms, 3),
                       "how": "the 64 instances one after another, each through MCState + "
                              "VMC_SR.advance (median-free mean of 2 steps after 1 warm-up)",
                       "speedup_of_batched": round(seq_ms / ms_max, 3)},
        "e2e": {"value": round(1000.0 / e2e_ms, 4), "unit": "steps/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 64 * 6 * 8},
        "solver_failures_last_step": bad,
        "gpu_launches": None, "clocks": clk.summary(),
    }


def run_serving(args):
    """Serving workload: a Poisson stream of expect_and_grad requests over a seeded
    mix of 1D TFIM (N 16-256) and 2D Heisenberg (6x6 .. 16x16) problems, alpha in
    {1, 2, 4}, 2048-16384 samples, swept over arrival rates; sessions stay
    resident on the device, admission by an HBM budget, 8 slots (streams).  The
    line reports p50 / p99 latency and throughput per rate and checks that
    requests give bit-identical results alone and in the mix."""
    import numpy as np
    import torch
    import netket_gb300 as nk

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    S = nk.serving
    specs = S.mixed_specs(48, seed=0)
    # warm-up: every session built and served once
    S.Server(hbm_budget_bytes=64 << 30, n_slots=8).serve(S.poisson_stream(specs, 1e4, seed=0))
    torch.cuda.synchronize()
    sweep = []
    with ClockSampler(local) as clk:
        for rate in (20.0, 50.0, 100.0, 200.0, 400.0):
            srv = S.Server(hbm_budget_bytes=64 << 30, n_slots=8)
            reqs = S.poisson_stream(specs, rate, seed=int(rate))
            t0 = time.perf_counter()
            res = srv.serve(reqs, t0=t0)
            wall = time.perf_counter() - t0
            row = S.latency_summary(res, wall)
            row.update(offered_rps=rate, peak_inflight=srv.peak_inflight)
            sweep.append(row)
    # alone vs mix on fresh servers (same sessions, same order)
    sub = specs[:6]
    alone = {}
    for k, spec in enumerate(sub):
        srv = S.Server(hbm_budget_bytes=64 << 30, n_slots=8)
        (r,) = srv.serve([S.Request(0.0, k, f"s{k}", spec, True)])
        alone[k] = r
    srv = S.Server(hbm_budget_bytes=64 << 30, n_slots=8)
    mix = {r.rid: r for r in srv.serve(S.poisson_stream(sub, 5000.0, seed=3))}
    same = all(np.array_equal(mix[k].stats.as_array(), alone[k].stats.as_array()) and
               np.array_equal(mix[k].grad, alone[k].grad) for k in alone)
    if rank != 0:
        return None
    top = max(sweep, key=lambda r: r["offered_rps"])
    return {
        "metric": "served expect_and_grad requests/s (p50/p99 ms)", "value": top["throughput_rps"],
        "unit": "requests/s", "n_gpus": world, "steps": len(specs), "warmup": 1,
        "ms_per_step": top["mean_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "serving_mix_48", "requests_per_rate": len(specs),
                   "mix": "TFIM N 16-256 / Heisenberg 6x6-16x16, alpha 1/2/4, 2048-16384 samples",
                   "slots": 8, "hbm_budget_gb": 64, "parallelism": f"replicas{world}"},
        "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"], "sweep": sweep,
        "alone_equals_mix": bool(same), "peak_inflight_in_mix": srv.peak_inflight,
        "e2e": {"value": top["throughput_rps"], "unit": "requests/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": None},
        "clocks": clk.summary(),
    }


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "source": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "source": "fallback"}


class CpuReference:
    """The reference algorithm on the host cores (numpy / scipy FP64, all host
    threads): ``oracle/vmc_step.py``'s step of the same 10x10 J1-J2 / alpha = 4
    workload at 16,384 samples, measured rather than modelled.  The
    per-sample phases (sampling, local energies, Jacobian rows, O_L^T aux) run on
    a slice of 128 chains x 4 samples (1/32 of the step's independent work), the
    Gram matrix as that slice's 512 rows of T against a full-size Jacobian, and
    the 16,384 x 16,384 Cholesky at full size once per run."""

    N_SLICE_CHAINS = 128

    def __init__(self, n_samples=16384, seed=0):
        import numpy as np
        from oracle import graph as og, hilbert as oh, operator as oop, rbm as orbm, vmc_step
        self.np, self.vmc_step = np, vmc_step
        g = og.Square(10, max_neighbor_order=2)
        op = oop.heisenberg(100, g, [1.0, 0.5], sign_rule=[True, False])
        self.tables = vmc_step.two_site_tables(op)
        clusters = np.sort(np.array(g.edges(), dtype=np.int64), axis=1)
        self.clusters = clusters[np.lexsort((clusters[:, 1], clusters[:, 0]))]
        self.rng = np.random.default_rng(seed)
        self.params = orbm.init_params(self.rng, 100, 4, 0.01)
        self.x = oh.random_state(self.rng, self.N_SLICE_CHAINS, 100, 0)
        self.n_samples = n_samples
        t0 = time.perf_counter()
        self.chol_s = vmc_step.full_size_cholesky_seconds(n_samples, 1e-4, self.rng)
        self.setup_s = time.perf_counter() - t0

    def step(self):
        """Seconds of one full-size step and its phases."""
        phases, reps = self.vmc_step.measured_full_step(
            self.params, self.x, self.rng, self.clusters, self.tables, 5, 4, 1e-4, 0.01,
            self.n_samples, self.chol_s)
        self.reps = reps
        return sum(phases.values()), phases

    def describe(self):
        return (f"every phase of the {self.n_samples}-sample step measured: sampling, local "
                f"energies, Jacobian rows and O_L^T aux on {self.N_SLICE_CHAINS} chains x 4 "
                f"samples (1/{self.reps} of the step's independent per-sample work, times "
                f"{self.reps}); T = O_L O_L^T as those 512 rows against a full-size "
                f"{self.n_samples} x 40500 FP64 Jacobian (times {self.reps}); the "
                f"{self.n_samples} x {self.n_samples} FP64 cho_factor + cho_solve at full size "
                f"({self.chol_s:.2f} s, timed once); numpy/scipy FP64 with {NPROC} host threads")


def run_cpu_baseline():
    ref = CpuReference()
    full_s, phases = ref.step()
    return {"value": round(1.0 / full_s, 6), "unit": "steps/s", "cores": NPROC, "kind": "port",
            "sample": ref.describe(),
            "phase_s": {k: round(v, 3) for k, v in phases.items()},
            "full_step_s": round(full_s, 3)}


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return None
    t_start = time.perf_counter()
    ref = CpuReference()
    for _ in range(args.warmup):
        ref.step()
    steps = []
    for _ in range(args.steps):
        steps.append(ref.step())
    full = [s for s, _ in steps]
    v = 1.0 / pystats.median(full)
    phases = {k: round(pystats.median(p[k] for _, p in steps), 3) for k in steps[0][1]}
    return {
        "impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": "steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000.0 / v, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(WORKLOAD, precision="fp64", parallelism="host cores"),
        "cpu_baseline": {"value": round(v, 6), "unit": "steps/s", "cores": NPROC, "kind": "port",
                         "sample": ref.describe()},
        "phase_s": phases,
        "e2e": {"value": round(v, 6), "unit": "steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": round(time.perf_counter() - t_start, 1),
        "note": "NetKet's JAX CPU path cannot be installed here (no jax/flax/optax/numba); "
                "the numpy FP64 restatement of the same algorithm is timed instead. Each "
                "step's value is the full-size step assembled from measured phases (see "
                "sample); wall_s is this process's own run time",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="minsr",
                    choices=["minsr", "batched", "serving", "large"],
                    help="minsr: the 10x10 J1-J2 step (the metric); batched: 64 TFIM "
                         "instances per step; serving: the request-stream sweep; large: the "
                         "16x16 alpha-8 step with 65,536 samples")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp32", "fp64"])
    ap.add_argument("--plain-steps", type=int, default=4)
    ap.add_argument("--n-chains", type=int, default=WORKLOAD["n_chains"],
                    help="smaller cases for profiling; the metric is quoted at the default")
    ap.add_argument("--n-samples", type=int, default=WORKLOAD["n_samples"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--gram-traffic", type=float, default=None)
    # DRAM bytes of one n = 16,384 solve, summed over its 537 launches in one ncu
    # capture (profiles/cholesky_solve_dram_n16384.md)
    ap.add_argument("--solve-traffic", type=float, default=15.72e9,
                    help="DRAM bytes of one solve (ncu); reported as roofline.traffic")
    ap.add_argument("--matched-steps", type=int, default=8,
                    help="steps of the matched-energy comparison (0 skips it)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        line = run_reference(args)
    elif args.workload == "batched":
        line = run_batched(args)
    elif args.workload == "serving":
        line = run_serving(args)
    else:
        line = run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

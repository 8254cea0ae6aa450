"""Benchmark: spin-slice updates/s of path-integral quantum annealing on the 80x80, P=20 workload.

Workload (per GPU): 80x80 periodic lattice, couplings iid N(0,1) rounded to FP32
(seeded synthetic instance), P = 20 Trotter slices, T = 0.05, transverse field
linear 3.0 -> 1e-8 over 2000 steps, 1 local sweep per step, 1024 replicas
started from random +-1 spins tiled over the slices.  One step = one complete
anneal of all replicas (2.62e11 spin-slice updates).

Arms:
  (default)          the packed CUDA kernel (libpiqmc_gb300.so).
                     value: device-timed throughput, inputs resident in HBM;
                     e2e: the same through piqmc.fast.anneal_replicas with host
                     buffers (H2D of the int8 configurations, D2H of the final
                     configurations and the FP64 energies inside the timed region).
  --impl reference   the reference's own Cython QuantumAnneal (compiled in
                     oracle/_ref; else the oracle's C port), one process per host
                     core, each annealing its own replica through a bounded sample
                     of the schedule (every 20th field value).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "pathintegral-qmc_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

from piqmc import shard  # noqa: E402  (replica sharding over ranks)

L_SIDE, P_SLICES, TEMP, NSCHED, REPLICAS = 80, 20, 0.05, 2000, 1024
FLOP_PER_UPDATE = 14   # 2(z+2)+2 FP32 flop per update at z = 4 (z coupling adds, 2 Trotter, x 1/T, exp)
METRIC = "spin-slice updates/s"


def schedule(nsched=NSCHED):
    return np.linspace(3.0, 1e-8, nsched)


# ------------------------------------------------------------------------------------------
# sharding over ranks: replicas only, no data-path collective
# ------------------------------------------------------------------------------------------

BENCH_SEED = 7


def rank_plan(rank, world, R):
    """Rank `rank` of `world` anneals the global replicas [rank R, (rank + 1) R) with the bench's key."""
    return shard.rank_plan(rank, world, R, BENCH_SEED)


initial_spins = shard.initial_spins
max_over_ranks = shard.max_over_ranks
whole_job_rate = shard.whole_job_rate


def instance_arrays(seed=2026):
    """Seeded 80x80 periodic N(0,1) instance: DOK keys in insertion order (right, down per spin)."""
    g = np.random.default_rng(seed)
    L = L_SIDE
    rows, cols, vals = [], [], []
    for y in range(L):
        for x in range(L):
            i = y * L + x
            rows += [i, i]
            cols += [y * L + (x + 1) % L, ((y + 1) % L) * L + x]
            vals += [float(np.float32(g.normal())), float(np.float32(g.normal()))]
    return np.array(rows), np.array(cols), np.array(vals)


def batched_instances(count=256, seed=2027):
    """Seeded uneven workload: L ~ U{8..48} periodic N(0,1) lattices, P ~ {16, 32, 64}, 8 replicas each."""
    g = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        L = int(g.integers(8, 49))
        P = int(g.choice([16, 32, 64]))
        n = L * L
        idx = np.arange(n)
        x, y = idx % L, idx // L
        rows = np.repeat(idx, 2)
        cols = np.stack([y * L + (x + 1) % L, ((y + 1) % L) * L + x], axis=1).ravel()
        vals = g.normal(size=2 * n).astype(np.float32).astype(np.float64)
        out.append((n, rows, cols, vals, P))
    return out


def neighbors_from_keys(n, rows, cols, vals, maxnb):
    """The (n, maxnb, 2) neighbour table in DOK key order, one pass over the keys (setup only)."""
    nbs = np.zeros((n, maxnb, 2))
    fill = np.zeros(n, dtype=np.int64)
    for a, b, v in zip(rows, cols, vals):
        nbs[a, fill[a]] = (b, v)
        fill[a] += 1
        if b != a:
            nbs[b, fill[b]] = (a, v)
            fill[b] += 1
    return nbs


# ------------------------------------------------------------------------------------------
# CPU baseline: the reference's QuantumAnneal, one process per core
# ------------------------------------------------------------------------------------------

def _ref_worker_init(use_ref):
    global _REF_QA, _NBS
    if use_ref:
        sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
        from piqmc_ref import qmc
        _REF_QA = ("reference", qmc.QuantumAnneal)
    else:
        import oracle
        _REF_QA = ("port", oracle)
    r, c, v = instance_arrays()
    _NBS = neighbors_from_keys(L_SIDE * L_SIDE, r, c, v, 4)


def _ref_worker_run(args):
    seed, sched = args
    n, P = L_SIDE * L_SIDE, P_SLICES
    g = np.random.default_rng(seed)
    conf0 = np.where(g.random(n) < 0.5, -1.0, 1.0)
    kind, fn = _REF_QA
    t0 = time.perf_counter()
    if kind == "reference":
        confs = np.tile(conf0, (P, 1)).T   # Fortran-ordered, as the reference's examples build it
        fn(sched, 1, P, TEMP, n, confs, _NBS, np.random.RandomState(seed))
    else:
        import oracle
        perms = oracle.reference_perms(np.random.RandomState(seed), n, len(sched))
        rands = g.integers(0, 2 ** 31 - 1, size=n * P * len(sched), dtype=np.int64).astype(np.int32)
        sp = np.ascontiguousarray(np.tile(conf0, (P, 1)).T.astype(np.int8))
        t0 = time.perf_counter()
        oracle.qa_sparse(sp, _NBS, sched, 1, TEMP, perms, rands)
    return time.perf_counter() - t0


def ref_available():
    import sysconfig
    d = os.path.join(ROOT, "oracle", "_ref", "piqmc_ref")
    return os.path.exists(os.path.join(d, "qmc" + sysconfig.get_config_var("EXT_SUFFIX")))


def cpu_baseline(steps, warmup, stride=20, cores=None):
    """Aggregate updates/s of the reference QuantumAnneal on all host cores (bounded sample)."""
    use_ref = ref_available()
    cores = cores or len(os.sched_getaffinity(0))
    sched = schedule()[::stride]
    ctx = mp.get_context("spawn")
    per = L_SIDE * L_SIDE * P_SLICES * len(sched)
    rates = []
    with ctx.Pool(cores, initializer=_ref_worker_init, initargs=(use_ref,)) as pool:
        for it in range(warmup + steps):
            t0 = time.perf_counter()
            pool.map(_ref_worker_run, [(1000 * it + c, sched) for c in range(cores)], chunksize=1)
            dt = time.perf_counter() - t0
            if it >= warmup:
                rates.append(per * cores / dt)
    return {"value": float(np.median(rates)), "unit": METRIC, "cores": cores,
            "kind": "reference" if use_ref else "port",
            "sample": "%d processes x 1 replica x 80x80x20 x %d field steps (every %dth of the 2000-step "
                      "schedule) per step; %s" % (cores, len(sched), stride,
                                                  "compiled reference Cython QuantumAnneal" if use_ref
                                                  else "oracle C port of QuantumAnneal")}


# ------------------------------------------------------------------------------------------
# clocks
# ------------------------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(statistics.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------

def measured_fp32_peak(torch):
    """FP32 FMA throughput of this GPU in TFLOP/s (in-run probe kernel of tests/native, best of 5)."""
    from piqmc import _device
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from native import probes
    lib = probes.lib()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4096
    out = torch.empty(blocks, device="cuda")
    best = 0.0
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lib.pqt_fp32_fma_probe(_device.ptr(out), iters, blocks, threads, _device.stream_handle())
        e1.record()
        torch.cuda.synchronize()
        best = max(best, blocks * threads * iters * 8 * 2 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def gpu_arm(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cpu_base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # spawn the CPU pool before any CUDA work
        cpu_base = cpu_baseline(steps=2, warmup=1)
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from piqmc import _native, fast

    lib = _native.lib()
    n, P, R = L_SIDE * L_SIDE, P_SLICES, args.replicas
    rows, cols, vals = instance_arrays()
    from piqmc import tools
    import scipy.sparse as sps
    J = sps.dok_matrix((n, n))
    for a, b, v in zip(rows, cols, vals):
        J[int(a), int(b)] = v
    nbs = tools.GenerateNeighbors(n, J, 4)
    prob = fast.Problem(nbs)
    sched = schedule(args.nsched)
    plan = rank_plan(rank, world, R)
    conf0 = initial_spins(plan["replica_base"], R, n)
    confs = np.ascontiguousarray(np.repeat(conf0[:, :, None], P, axis=2))
    words0 = prob.pack(torch.from_numpy(confs))
    words = words0.clone()
    jp = torch.from_numpy(fast.jperp_schedule(sched, P, TEMP)).cuda()
    status = fast._device.Status()
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    seed0 = plan["seed"]
    updates = float(n) * P * R * len(sched)

    def one_step(it):
        fast.anneal(prob, words, sched, P, TEMP, seed=seed0 + it, jperp=jp, status=status, check=False,
                    threads=args.threads, replicas_per_cta=args.rpc, replica_base=plan["replica_base"])

    for it in range(args.warmup):
        words.copy_(words0)
        one_step(it)
    status.raise_if_set("warmup")
    times = []
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for it in range(args.steps):
            words.copy_(words0)
            l2_flush.fill_(float(it))          # write > L2 between timed iterations
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            one_step(args.warmup + it)
            e1.record()
            times.append((e0, e1))
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    status.raise_if_set("timed steps")
    step_ms = [a.elapsed_time(b) for a, b in times]
    total_s = sum(step_ms) * 1e-3
    if world > 1:
        total_s = max_over_ranks(total_s, dist, "cuda")
    value = whole_job_rate(updates, args.steps, world, total_s)
    # energies of the last anneal: residual-energy summary (per spin, best slice)
    E = prob.energies(words, P).cpu().numpy()
    best = E.min(axis=1) / n

    # e2e through the host-buffer API
    pinned_in = torch.from_numpy(confs).pin_memory()
    out_c = torch.empty((R, n, P), dtype=torch.int8, pin_memory=True)
    out_e = torch.empty((R, P), dtype=torch.float64, pin_memory=True)
    fast.anneal_replicas(prob, pinned_in, sched, P, TEMP, seed=seed0, out=out_c, energies_out=out_e,
                         replica_base=plan["replica_base"])
    e2e_ms = []
    for it in range(max(1, min(args.steps, 3))):
        l2_flush.fill_(float(it))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fast.anneal_replicas(prob, pinned_in, sched, P, TEMP, seed=seed0 + 100 + it, out=out_c, energies_out=out_e,
                             replica_base=plan["replica_base"])
        e1.record()
        torch.cuda.synchronize()
        e2e_ms.append(e0.elapsed_time(e1))
    e2e_s = sum(e2e_ms) * 1e-3
    if world > 1:
        e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    e2e_value = whole_job_rate(updates, len(e2e_ms), world, e2e_s)

    batched = densew = learnedw = reforderw = dropinw = genw = None
    if not args.no_batched and rank == 0:
        batched = batched_workload(args, torch)
        densew = dense_workload(args, torch)
        learnedw = learned_vs_plain(args, torch, prob, R=args.learned_replicas)
        reforderw = reforder_workload(args, torch)
        dropinw = dropin_workload(args, torch)
        genw = generators_workload(args, torch)

    peak = measured_fp32_peak(torch)
    achieved_tflops = value / world * FLOP_PER_UPDATE / 1e12
    ms_per_step = total_s / args.steps * 1e3
    traffic, issue = None, None
    prof = os.path.join(ROOT, "profiles", "qa_fast_kernel_80x80_P20.traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as f:
                pj = json.load(f)
            traffic = pj.get("dram_bytes_per_launch")
            issue = pj.get("issue")
        except (OSError, ValueError):
            traffic = None
    clocks = clk.summary()
    if issue and issue.get("instructions_per_update"):
        # the instruction-issue roof: 4 warp instructions per cycle per SM at the sampled SM clock
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
        if mhz:
            roof = sms * 4 * 32 * mhz * 1e6 / issue["instructions_per_update"]
            issue = dict(issue, issue_roof_updates_per_s=roof, issue_frac=(value / world) / roof)
    line = {
        "metric": METRIC, "value": value, "unit": "updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": "80x80 periodic lattice, J~N(0,1) fp32, P=20, T=0.05, G linear 3.0->1e-8 over "
                               "%d steps, %d replicas/GPU, 1 local sweep/step, packed kernel, random class order"
                               % (len(sched), R),
                   "replicas_per_gpu": R, "spins": n, "slices": P, "field_steps": len(sched),
                   "updates_per_step": updates * world, "parallelism": "replicas%d" % world,
                   "l2": "256 MB buffer written between timed steps"},
        "e2e": {"value": e2e_value, "unit": "updates/s", "h2d_bytes_per_step": int(confs.nbytes),
                "d2h_bytes_per_step": int(out_c.numel() + out_e.numel() * 8)},
        "gpu_launches": args.steps,
        "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved_tflops / peak, "traffic": traffic,
                     "note": "achieved = %d FP32 flop per spin-slice update x updates/s of the packed sweep "
                             "(qa_fast_kernel, one launch per step, CUDA events); peak = in-run FP32 FMA probe "
                             "(no FP32 figure in the measured-peaks file)" % FLOP_PER_UPDATE,
                     "binding_unit": issue},
        "clocks": clocks,
        "residual": {"best_slice_energy_per_spin_median": float(np.median(best)),
                     "best_slice_energy_per_spin_min": float(best.min())},
        "wall_s_timed": wall,
    }
    if cpu_base is not None:
        line["cpu_baseline"] = cpu_base
    extras = compact_extras(batched, densew, learnedw, reforderw, dropinw, genw)
    if extras:
        # the compact figures go right after the config, the detailed objects at the end of the line
        keys = list(line)
        at = keys.index("config") + 1
        line = {k: line[k] for k in keys[:at]} | {"extras": extras} | {k: line[k] for k in keys[at:]}
    if dropinw is not None:
        line["dropin"] = dropinw
    if genw is not None:
        line["generators"] = genw
    if batched is not None:
        line["batched_uneven"] = batched
    if densew is not None:
        line["dense"] = densew
    if learnedw is not None:
        line["learned_vs_uniform"] = learnedw
    if reforderw is not None:
        line["reference_order"] = reforderw
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def compact_extras(batched, densew, learnedw, reforderw, dropinw, genw=None):
    """Headline figure of every extra workload, in a few keys (the detailed objects follow at the end)."""
    ex = {}
    if batched is not None:
        ex["batched_uneven_updates_per_s"] = batched["value"]
    if densew is not None:
        ex["dense_N512_P32_updates_per_s"] = densew["value"]
        if "cpu_baseline" in densew:
            ex["dense_reference_all_cores_updates_per_s"] = densew["cpu_baseline"]["value"]
    if learnedw is not None:
        ex["learned_time_to_plain_residual_over_plain"] = learnedw.get("learned_time_to_plain_residual_over_plain")
        ex["uniform_pair_time_to_plain_residual_over_plain"] = learnedw.get(
            "uniform_pair_time_to_plain_residual_over_plain")
    if reforderw is not None:
        ex["reference_order_1_replica_updates_per_s"] = reforderw["replicas_1"]["value"]
        ex["reference_order_8_replicas_updates_per_s"] = reforderw["replicas_8"]["value"]
    if dropinw is not None:
        ex["dropin_speedup_vs_one_core"] = {r["call"].split(" ")[0]: r.get("speedup_vs_one_core")
                                            for r in dropinw["calls"]}
    if genw is not None:
        ex["generator_gpu_ms"] = {r["instance"]: r["gpu_ms"] for r in genw["instances"]}
    return ex


def batched_workload(args, torch):
    """The uneven batched workload through one persistent launch per anneal, replayed as a CUDA graph."""
    from piqmc import autotune, batch
    insts = batched_instances(args.batched_count)
    nbs_list = [neighbors_from_keys(n, r, c, v, 4) for n, r, c, v, _ in insts]
    P = [p for *_, p in insts]
    R = [8] * len(insts)
    t0 = time.perf_counter()
    B = batch.Batch(nbs_list, R, P, tuner=autotune.tune)
    tune_s = time.perf_counter() - t0
    g = np.random.default_rng(5)
    spins = [np.repeat(np.where(g.random((8, n)) < 0.5, -1, 1).astype(np.int8)[:, :, None], p, axis=2)
             for (n, *_), p in zip(insts, P)]
    sched = schedule(args.batched_steps)
    B.set_spins(spins)
    B.anneal(sched, TEMP, seed=1, graph=True, chunk=100)          # eager run + capture
    updates = float(sum(n * p * 8 for (n, *_), p in zip(insts, P))) * len(sched)
    times = []
    for it in range(max(2, min(args.steps, 3))):
        B.set_spins(spins)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        B.anneal(sched, TEMP, seed=1, graph=True, chunk=100)      # graph replay
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    best = [float(e.min().item()) for e in B.energies()]
    return {"workload": "%d instances, L~U{8..48} periodic, J~N(0,1) fp32, P~{16,32,64}, 8 replicas each, "
                        "T=0.05, G 3.0->1e-8 over %d steps; one persistent launch per 100 steps, graph-replayed"
                        % (len(insts), len(sched)),
            "value": updates / float(np.median(times)), "unit": "updates/s", "ms_per_anneal": 1e3 * float(np.median(times)),
            "updates_per_anneal": updates, "tasks": int(len(B.tasks)), "grid": int(B.grid),
            "tiles": sorted(set(map(tuple, B.tiles))), "tune_s": tune_s,
            "ms_per_field_step": 1e3 * float(np.median(times)) / len(sched),
            "tuner_predicted_ms_per_field_step": 1e3 * getattr(B, "predicted_step_s", float("nan")),
            "best_energy_sum": float(sum(best))}


def dense_instance(N=512, seed=2028):
    """Seeded dense instance: J_ij ~ N(0, 1/N) on the upper triangle (fp32 values), fields ~ N(0, 0.1)."""
    g = np.random.default_rng(seed)
    J = np.triu(g.normal(0.0, 1.0 / np.sqrt(N), (N, N)).astype(np.float32).astype(np.float64), 1)
    J += np.diag(g.normal(0.0, np.sqrt(0.1), N).astype(np.float32).astype(np.float64))
    return J


def _dense_ref_worker(args):
    seed, steps = args
    sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
    from piqmc_ref import qmc
    J = dense_instance()
    N, P = J.shape[0], 32
    g = np.random.default_rng(seed)
    confs = np.tile(np.where(g.random(N) < 0.5, -1.0, 1.0), (P, 1)).T
    t0 = time.perf_counter()
    qmc.QuantumAnneal_dense(schedule(1000)[::1000 // steps][:steps], 1, P, TEMP, N, confs, J, np.random.RandomState(seed))
    return time.perf_counter() - t0


def dense_workload(args, torch):
    """Dense N=512, P=32, 256 replicas, 1000 field steps: split-BF16 tcgen05 field recompute every 50 steps."""
    from piqmc import dense
    J = dense_instance()
    N, P, R = J.shape[0], 32, args.dense_replicas
    prob = dense.DenseProblem(J)
    g = np.random.default_rng(9)
    spins = np.repeat(np.where(g.random((R, N)) < 0.5, -1, 1).astype(np.int8)[:, :, None], P, axis=2)
    w0 = prob.pack(torch.from_numpy(spins))
    sched = schedule(args.dense_steps)
    w = w0.clone()
    prob.anneal(w, sched[:50], P, TEMP, seed=1)
    torch.cuda.synchronize()
    times = []
    for it in range(2):
        w = w0.clone()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        prob.anneal(w, sched, P, TEMP, seed=2 + it, recompute_every=50)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    err, scale = dense.field_error(prob, w, P)
    E = prob.energies(w, P).cpu().numpy()
    updates = float(N) * P * R * len(sched)
    out = {"workload": "dense N=512, J~N(0,1/N) fp32, h~N(0,0.1), P=32, T=0.05, G 3.0->1e-8 over %d steps, "
                       "%d replicas; fields recomputed every 50 steps by the split-BF16 tcgen05 GEMM" % (len(sched), R),
           "value": updates / min(times), "unit": "updates/s", "ms_per_anneal": 1e3 * min(times),
           "field_recompute_max_abs_error_vs_fp64": err, "field_max_abs": scale,
           "best_energy_per_spin_median": float(np.median(E.min(axis=1)) / N)}
    if ref_available() and not args.no_cpu_baseline:
        cores = len(os.sched_getaffinity(0))
        steps = 4
        with mp.get_context("spawn").Pool(cores) as pool:
            pool.map(_dense_ref_worker, [(c, 1) for c in range(cores)])
            t0 = time.perf_counter()
            pool.map(_dense_ref_worker, [(100 + c, steps) for c in range(cores)])
            wall = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": N * P * steps * cores / wall, "unit": "updates/s", "cores": cores,
                               "kind": "reference",
                               "sample": "%d processes x QuantumAnneal_dense N=512 P=32 x %d field steps" % (cores, steps)}
    return out


def learned_vs_plain(args, torch, prob_big, R=1024, every=20):
    """Residual energy at equal GPU time on the 80x80 P=20 workload: plain vs pair forms.

    Forms (the same local sweeps; a move pass every `every` field steps):
      plain         uniform single world-line moves (every spin tried) -- the method the others are judged by;
      uniform_pair  plain + a pair world-line pass that tries every bond (piqmc.pairs.pair_pass);
      learned_pair  plain + pair moves proposed by the MLP (8 -> 64 -> 64 -> 1, BF16 on the tensor cores)
                    with the exact Metropolis-Hastings correction (piqmc.pairs.learned_pair_pass), trained
                    on pair moves recorded from uniform-pair runs of a 32x32 P=20 instance (J ~ U[-2, 2]).
    Residual energy per spin = best-slice energy minus the best energy any run found, over n.  The target
    is the plain form's median at the full 2000-step schedule; a form's time to it is the GPU time of its
    shortest schedule whose median reaches it."""
    import scipy.sparse as sps
    from piqmc import fast, learned, pairs, tools
    P = P_SLICES
    g = np.random.default_rng(11)
    L = 32
    J = sps.dok_matrix((L * L, L * L))
    for y in range(L):
        for x in range(L):
            i = y * L + x
            J[i, y * L + (x + 1) % L] = float(np.float32(g.uniform(-2, 2)))
            J[i, ((y + 1) % L) * L + x] = float(np.float32(g.uniform(-2, 2)))
    small = fast.Problem(tools.GenerateNeighbors(L * L, J, 4))
    Rs = 64
    sched_s = schedule(200)
    jp_s = fast.jperp_schedule(sched_s, P, TEMP)
    spins_s = np.repeat(np.where(g.random((Rs, L * L)) < 0.5, -1, 1).astype(np.int8)[:, :, None], P, axis=2)
    ws = small.pack(torch.from_numpy(spins_s))
    t0 = time.perf_counter()
    Xs, ys = [], []
    for g0 in range(0, len(sched_s), 20):
        fast.anneal(small, ws, sched_s[g0:g0 + 20], P, TEMP, seed=21, sweep_base=g0,
                    jperp=torch.from_numpy(jp_s[g0:g0 + 20]).cuda())
        X, y = pairs.record_pair_moves(small, ws, P, 1.0 / TEMP, float(jp_s[g0 + 19]))
        Xs.append(X)
        ys.append(y)
        pairs.pair_pass(small, ws, P, 1.0 / TEMP, seed=22, move=g0)
    X, y = torch.cat(Xs), torch.cat(ys)
    mlp = learned.ProposalMLP(seed=0)
    hist = mlp.train(X, y, epochs=2, batch=16384, lr=3e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    n = prob_big.n
    spins = np.repeat(np.where(np.random.default_rng(12).random((R, n)) < 0.5, -1, 1).astype(np.int8)[:, :, None], P,
                      axis=2)
    pairs.bond_classes(prob_big)

    def run(kind, steps):
        sched = schedule(steps)
        jp_host = fast.jperp_schedule(sched, P, TEMP)
        jp = torch.from_numpy(jp_host).cuda()
        w = prob_big.pack(torch.from_numpy(spins))
        cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        pcnt = torch.zeros(2, dtype=torch.int64, device="cuda")
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        marks = []
        e0.record()
        for g0 in range(0, len(sched), every):
            g1 = min(len(sched), g0 + every)
            fast.anneal(prob_big, w, sched[g0:g1], P, TEMP, seed=31, sweep_base=g0, jperp=jp[g0:g1], check=False)
            pa, pb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            pa.record()
            learned.learned_pass(prob_big, w, P, None, 1.0 / TEMP, float(jp_host[g1 - 1]), seed=32, move=g0,
                                 counters=cnt, uniform=True, check=False)
            if kind == "uniform_pair":
                pairs.pair_pass(prob_big, w, P, 1.0 / TEMP, seed=33, move=g0, counters=pcnt, status=status,
                                check=False)
            elif kind == "learned_pair":
                pairs.learned_pair_pass(prob_big, w, P, mlp, 1.0 / TEMP, float(jp_host[g1 - 1]), seed=33, move=g0,
                                        counters=pcnt, status=status, check=False)
            pb.record()
            marks.append((pa, pb))
        e1.record()
        torch.cuda.synchronize()
        if int(status.item()):
            raise RuntimeError("pair pass status %d" % int(status.item()))
        E = prob_big.energies(w, P).cpu().numpy().min(axis=1)
        c, pc = cnt.cpu().numpy(), pcnt.cpu().numpy()
        return {"gpu_s": e0.elapsed_time(e1) * 1e-3, "best": E, "wl_tried": int(c[0]), "wl_accepted": int(c[1]),
                "pair_tried": int(pc[0]), "pair_accepted": int(pc[1]),
                "pass_ms": sum(a.elapsed_time(b) for a, b in marks) / len(marks)}

    plan = {"plain": (2000, 1400, 1000, 700), "uniform_pair": (400, 200, 100, 50), "learned_pair": (400, 200, 100, 50)}
    res = {(kind, st): run(kind, st) for kind, lens in plan.items() for st in lens}
    e_ref = min(r["best"].min() for r in res.values())
    plain = res[("plain", 2000)]
    target = float(np.median(plain["best"] - e_ref) / n)
    out = {"workload": "80x80 P=20, %d replicas, a move pass every %d steps; plain (single world-line moves) at %s "
                       "steps, uniform and learned pair world-line moves at %s steps; MLP 8-64-64-1 trained on pair "
                       "moves recorded from uniform-pair 32x32 P=20 runs"
                       % (R, every, "/".join(map(str, plan["plain"])), "/".join(map(str, plan["learned_pair"]))),
           "train_s": train_s, "train_rows": int(X.shape[0]), "train_loss_first_last": [hist[0], hist[-1]],
           "plain_median_residual_energy_per_spin": target, "runs": []}
    for (kind, st), r in res.items():
        out["runs"].append({"form": kind, "steps": st, "gpu_s": r["gpu_s"],
                            "median_residual_energy_per_spin": float(np.median(r["best"] - e_ref) / n),
                            "worldline_tried": r["wl_tried"], "worldline_accepted": r["wl_accepted"],
                            "pair_tried": r["pair_tried"], "pair_accepted": r["pair_accepted"],
                            "ms_per_move_pass": r["pass_ms"]})

    def time_to_target(kind):
        hits = [r for r in out["runs"] if r["form"] == kind and r["median_residual_energy_per_spin"] <= target]
        return min(r["gpu_s"] for r in hits) if hits else None

    tl, tu = time_to_target("learned_pair"), time_to_target("uniform_pair")
    out["learned_time_to_plain_residual_over_plain"] = tl / plain["gpu_s"] if tl else None
    out["uniform_pair_time_to_plain_residual_over_plain"] = tu / plain["gpu_s"] if tu else None
    out["learned_over_uniform_pair_time_to_target"] = tl / tu if tl and tu else None
    return out


def reforder_workload(args, torch):
    """Reference-order sweeps (the drop-in's bit-exact mode) on the 32x32 periodic P=20 lattice.

    8 replicas (and 1) with synthetic permutations and uniform streams in the
    reference's formats, one launch each, timed with CUDA events; the same kernel
    the drop-in QuantumAnneal runs (exp close calls are not resolved here)."""
    from piqmc import _device, _native, reforder, tools
    import scipy.sparse as sps
    L, P, steps = 32, 20, args.reforder_steps
    n = L * L
    g = np.random.default_rng(17)
    J = sps.dok_matrix((n, n))
    for y in range(L):
        for x in range(L):
            i = y * L + x
            J[i, y * L + (x + 1) % L] = float(np.float32(g.uniform(-2, 2)))
            J[i, ((y + 1) % L) * L + x] = float(np.float32(g.uniform(-2, 2)))
    nbs = tools.GenerateNeighbors(n, J, 4)
    idx, jv = reforder.split_neighbors(nbs)
    sched = schedule(steps)
    jp = torch.from_numpy(reforder.jperp_schedule(sched, P, TEMP)).cuda()
    lib = _native.lib()
    out = {"workload": "32x32 periodic, J~U[-2,2] fp32, P=20, T=0.05, %d steps, reference order (bit-exact mode), "
                       "synthetic permutations and uniform streams" % steps}
    for R in (1, 8):
        perms = torch.from_numpy(np.stack([np.stack([g.permutation(n) for _ in range(steps)]) for _ in range(R)])
                                 .astype(np.int32)).cuda()
        cap = n * P * steps
        rands = torch.from_numpy(g.integers(0, 2 ** 31 - 1, size=(R, cap), dtype=np.int64).astype(np.int32)).cuda()
        spins0 = torch.from_numpy(np.repeat(np.where(g.random((R, n)) < 0.5, -1, 1).astype(np.int8)[:, :, None], P,
                                            axis=2)).cuda()
        d_idx, d_j = torch.from_numpy(idx).cuda(), torch.from_numpy(jv).cuda()
        used = torch.zeros(R, dtype=torch.int64, device="cuda")
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        times = []
        for it in range(3):
            sp = spins0.clone()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            rc = lib.pq_qa_sparse_reforder(_device.ptr(sp), _device.ptr(d_idx), _device.ptr(d_j), n, n, idx.shape[1],
                                           P, R, _device.ptr(jp), steps, 1, float(np.float32(TEMP)),
                                           _device.ptr(perms), _device.ptr(rands), cap, _device.ptr(used), 0,
                                           _device.ptr(status), _device.stream_handle())
            e1.record()
            torch.cuda.synchronize()
            _native.check(rc, "pq_qa_sparse_reforder")
            if int(status.item()) or int(used.min().item()) < 0:
                raise RuntimeError("reference-order bench: status %d" % int(status.item()))
            times.append(e0.elapsed_time(e1) * 1e-3)
        out["replicas_%d" % R] = {"value": float(n) * P * steps * R / min(times), "unit": "updates/s",
                                  "ms": 1e3 * min(times)}
    # the same sweep on the headline's 80x80 instance (P = 20), one replica, 20 field steps
    n80 = L_SIDE * L_SIDE
    r80, c80, v80 = instance_arrays()
    i80, j80 = reforder.split_neighbors(neighbors_from_keys(n80, r80, c80, v80, 4))
    s80 = schedule(NSCHED)[:: NSCHED // 20][:20]
    jp80 = torch.from_numpy(reforder.jperp_schedule(s80, P, TEMP)).cuda()
    perms = torch.from_numpy(np.stack([g.permutation(n80) for _ in range(len(s80))])[None].astype(np.int32)).cuda()
    cap = n80 * P * len(s80)
    rands = torch.from_numpy(g.integers(0, 2 ** 31 - 1, size=(1, cap), dtype=np.int64).astype(np.int32)).cuda()
    sp0 = torch.from_numpy(np.repeat(np.where(g.random((1, n80)) < 0.5, -1, 1).astype(np.int8)[:, :, None], P,
                                     axis=2)).cuda()
    d_i80, d_j80 = torch.from_numpy(i80).cuda(), torch.from_numpy(j80).cuda()
    used = torch.zeros(1, dtype=torch.int64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    times = []
    for it in range(2):
        sp = sp0.clone()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = lib.pq_qa_sparse_reforder(_device.ptr(sp), _device.ptr(d_i80), _device.ptr(d_j80), n80, n80,
                                       i80.shape[1], P, 1, _device.ptr(jp80), len(s80), 1, float(np.float32(TEMP)),
                                       _device.ptr(perms), _device.ptr(rands), cap, _device.ptr(used), 0,
                                       _device.ptr(status), _device.stream_handle())
        e1.record()
        torch.cuda.synchronize()
        _native.check(rc, "pq_qa_sparse_reforder")
        if int(status.item()) or int(used.min().item()) < 0:
            raise RuntimeError("reference-order 80x80 bench: status %d" % int(status.item()))
        times.append(e0.elapsed_time(e1) * 1e-3)
    out["replicas_1_80x80"] = {"value": float(n80) * P * len(s80) / min(times), "unit": "updates/s",
                               "ms": 1e3 * min(times),
                               "workload": "80x80 periodic, J~N(0,1) fp32, P=20, 20 field steps, reference order"}
    # sa.Anneal's reference-order sweep, one replica, 100 temperatures 5 -> 0.05
    temps = torch.from_numpy(np.linspace(5.0, 0.05, steps).astype(np.float32)).cuda()
    perms = torch.from_numpy(np.stack([g.permutation(n) for _ in range(steps)])[None].astype(np.int32)).cuda()
    rands = torch.from_numpy(g.integers(0, 2 ** 31 - 1, size=(1, n * steps), dtype=np.int64).astype(np.int32)).cuda()
    s0 = torch.from_numpy(np.where(g.random((1, n)) < 0.5, -1, 1).astype(np.int8)).cuda()
    d_idx, d_j = torch.from_numpy(idx).cuda(), torch.from_numpy(jv).cuda()
    used = torch.zeros(1, dtype=torch.int64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    times = []
    for it in range(3):
        sp = s0.clone()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = lib.pq_sa_sparse_reforder(_device.ptr(sp), _device.ptr(d_idx), _device.ptr(d_j), n, idx.shape[1], 1,
                                       _device.ptr(temps), steps, 1, _device.ptr(perms), _device.ptr(rands), n * steps,
                                       _device.ptr(used), _device.ptr(status), _device.stream_handle())
        e1.record()
        torch.cuda.synchronize()
        _native.check(rc, "pq_sa_sparse_reforder")
        if int(status.item()) or int(used.min().item()) < 0:
            raise RuntimeError("reference-order SA bench: status %d" % int(status.item()))
        times.append(e0.elapsed_time(e1) * 1e-3)
    out["sa_replicas_1"] = {"value": float(n) * steps / min(times), "unit": "updates/s", "ms": 1e3 * min(times)}
    # QuantumAnneal_dense's reference-order sweep on the dense workload's instance (N = 512, P = 32)
    Jd = dense_instance()
    nd, Pd = Jd.shape[0], 32
    d_Jd = torch.from_numpy(Jd).cuda()
    for R, dsteps in ((1, 4), (256, 2)):
        dsched = schedule(1000)[:dsteps]
        jpd = torch.from_numpy(reforder.jperp_schedule(dsched, Pd, TEMP)).cuda()
        perms = torch.from_numpy(np.stack([np.stack([g.permutation(nd) for _ in range(dsteps)]) for _ in range(R)])
                                 .astype(np.int32)).cuda()
        cap = nd * Pd * dsteps
        rands = torch.from_numpy(g.integers(0, 2 ** 31 - 1, size=(R, cap), dtype=np.int64).astype(np.int32)).cuda()
        s0 = torch.from_numpy(np.repeat(np.where(g.random((R, nd)) < 0.5, -1, 1).astype(np.int8)[:, :, None], Pd,
                                        axis=2)).cuda()
        used = torch.zeros(R, dtype=torch.int64, device="cuda")
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        times = []
        for it in range(2):
            sp = s0.clone()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            rc = lib.pq_qa_dense_reforder(_device.ptr(sp), _device.ptr(d_Jd), nd, Pd, R, _device.ptr(jpd), dsteps, 1,
                                          float(np.float32(TEMP)), _device.ptr(perms), _device.ptr(rands), cap,
                                          _device.ptr(used), 0, _device.ptr(status), _device.stream_handle())
            e1.record()
            torch.cuda.synchronize()
            _native.check(rc, "pq_qa_dense_reforder")
            if int(status.item()) or int(used.min().item()) < 0:
                raise RuntimeError("reference-order dense bench: status %d" % int(status.item()))
            times.append(e0.elapsed_time(e1) * 1e-3)
        out["dense_replicas_%d" % R] = {"value": float(nd) * Pd * dsteps * R / min(times), "unit": "updates/s",
                                        "ms": 1e3 * min(times),
                                        "workload": "dense N=512, P=32, %d field steps, reference order" % dsteps}
    # sa.Anneal_bipartite's reference-order sweep: 512 + 512 spins, J ~ N(0, 1/512), biases ~ N(0, 0.1), FP64
    nl = nr = 512
    Jb = torch.from_numpy(g.normal(0.0, 1.0 / np.sqrt(nl), (nl, nr))).cuda()
    lb = torch.from_numpy(g.normal(0.0, 0.1, nl)).cuda()
    rb = torch.from_numpy(g.normal(0.0, 0.1, nr)).cuda()
    for R, bsteps in ((1, 4), (256, 2)):
        btemps = torch.from_numpy(np.linspace(3.0, 0.05, bsteps).astype(np.float32)).cuda()
        cap = (nl + nr) * bsteps
        rands = torch.from_numpy(g.integers(0, 2 ** 31 - 1, size=(R, cap), dtype=np.int64).astype(np.int32)).cuda()
        s0 = torch.from_numpy(np.where(g.random((R, nl + nr)) < 0.5, -1, 1).astype(np.int8)).cuda()
        used = torch.zeros(R, dtype=torch.int64, device="cuda")
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        times = []
        for it in range(2):
            sp = s0.clone()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            rc = lib.pq_sa_bipartite_reforder_ex(_device.ptr(sp), _device.ptr(Jb), nl, nr, _device.ptr(lb),
                                                 _device.ptr(rb), R, _device.ptr(btemps), bsteps, 1, _device.ptr(rands),
                                                 cap, _device.ptr(used), None, None, 0, None, None, 0, None,
                                                 _device.ptr(status), _device.stream_handle())
            e1.record()
            torch.cuda.synchronize()
            _native.check(rc, "pq_sa_bipartite_reforder_ex")
            if int(status.item()) or int(used.min().item()) < 0:
                raise RuntimeError("reference-order bipartite bench: status %d" % int(status.item()))
            times.append(e0.elapsed_time(e1) * 1e-3)
        out["bipartite_replicas_%d" % R] = {"value": float(nl + nr) * bsteps * R / min(times), "unit": "updates/s",
                                            "ms": 1e3 * min(times),
                                            "workload": "sa.Anneal_bipartite 512+512, FP64 weights, %d steps" % bsteps}
    return out


def gemm_workload(args, torch):
    """The tcgen05/TMA GEMM (pq_tc_gemm_bf16) alone: the dense recompute's shape and two large ones.

    Ten back-to-back calls between CUDA events (the launches queue, so host-side
    tensor-map encoding is hidden); checked against torch's product of the same BF16
    operands; cuBLAS timed beside it for reference."""
    from piqmc.tensor import gemm_bf16
    torch.manual_seed(0)
    out = {"workload": "D = A B^T, BF16 operands, FP32 accumulate and output", "shapes": []}
    for (M, N, K) in [(8192, 512, 1024), (8192, 8192, 8192), (16384, 4096, 4096)]:
        A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
        B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
        D = torch.empty(M, N, device="cuda")
        for _ in range(3):
            gemm_bf16(A, B, out=D)
        torch.cuda.synchronize()
        from piqmc.tensor import check_status

        def timed(fn):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(10):
                fn()
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) * 1e-3 / 10

        t = min(timed(lambda: gemm_bf16(A, B, out=D, check=False)) for _ in range(3))
        check_status()
        tc = min(timed(lambda: torch.matmul(A, B.T)) for _ in range(3))
        ref = A[:256].float() @ B.float().T
        err = float((D[:256] - ref).abs().max().item())
        out["shapes"].append({"M": M, "N": N, "K": K, "us": t * 1e6, "tflops": 2.0 * M * N * K / t / 1e12,
                              "cublas_us": tc * 1e6, "max_abs_err_vs_fp32_product": err})
    return out


def dropin_workload(args, torch):
    """The default drop-in calls end to end, as an existing script makes them: reference order, one replica per
    call, host buffers in and out, the permutations drawn from the caller's rng and the uniforms from this
    process's libc rand() inside the timed call.  Each beside the compiled reference's own call on one host
    core (oracle/_ref), same inputs; updates/s = spins x slices x field steps x mcsteps / wall time."""
    from piqmc import qmc as d_qmc, sa as d_sa, tools
    import scipy.sparse as sps
    ref = None
    if ref_available():
        sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
        from piqmc_ref import qmc as r_qmc, sa as r_sa
        ref = (r_qmc, r_sa)
    g = np.random.default_rng(31)

    def timed(fn, *a):
        t0 = time.perf_counter()
        fn(*a)
        return time.perf_counter() - t0

    out = {"note": "wall time of one synchronous call (host streams, copies and the kernel); reference: the "
                   "compiled reference's same call on one host core"}
    # QuantumAnneal: the headline 80x80 P=20 instance, 20 field values of its schedule
    n, P = L_SIDE * L_SIDE, P_SLICES
    rows, cols, vals = instance_arrays()
    J = sps.dok_matrix((n, n))
    for a_, b_, v in zip(rows, cols, vals):
        J[int(a_), int(b_)] = v
    nbs = tools.GenerateNeighbors(n, J, 4)
    conf0 = np.tile(np.where(g.random(n) < 0.5, -1.0, 1.0), (P, 1)).T
    sched = schedule()[::100]
    cases = [("QuantumAnneal 80x80 P=20, %d field steps" % len(sched), n * P * len(sched),
              lambda m: (lambda: m.QuantumAnneal(sched, 1, P, TEMP, n, conf0.copy(order="F"), nbs,
                                                 np.random.RandomState(1))))]
    # QuantumAnneal_dense: N=512, P=32, FP64-valued couplings (a user's np.random matrix), 4 field steps
    N, Pd = 512, 32
    Jd = np.triu(g.normal(0.0, 1.0 / np.sqrt(N), (N, N)), 1) + np.diag(g.normal(0.0, np.sqrt(0.1), N))
    confd = np.tile(np.where(g.random(N) < 0.5, -1.0, 1.0), (Pd, 1)).T
    schedd = schedule(1000)[::250]
    cases.append(("QuantumAnneal_dense N=512 P=32 FP64-valued J, %d field steps" % len(schedd), N * Pd * len(schedd),
                  lambda m: (lambda: m.QuantumAnneal_dense(schedd, 1, Pd, TEMP, N, confd.copy(order="F"), Jd,
                                                           np.random.RandomState(2)))))
    # sa.Anneal: the 80x80 instance, classical, 50 temperatures
    temps = np.linspace(3.0, 0.05, 50)
    sv0 = np.where(g.random(n) < 0.5, -1.0, 1.0)
    cases.append(("sa.Anneal 80x80, %d temperatures" % len(temps), n * len(temps),
                  lambda m: (lambda: m.Anneal(temps, 1, sv0.copy(), nbs, np.random.RandomState(3)))))
    # sa.Anneal_bipartite: 256 + 256 spins, FP64-valued couplings and biases, 20 temperatures
    nl = nr = 256
    Jb = g.normal(0.0, 1.0 / np.sqrt(nl), (nl, nr))
    lb, rb = g.normal(0.0, 0.3, nl), g.normal(0.0, 0.3, nr)
    lv0, rv0 = np.where(g.random(nl) < 0.5, -1.0, 1.0), np.where(g.random(nr) < 0.5, -1.0, 1.0)
    tb = np.linspace(3.0, 0.05, 20)
    cases.append(("sa.Anneal_bipartite 256+256 FP64-valued J, %d temperatures" % len(tb), (nl + nr) * len(tb),
                  lambda m: (lambda: m.Anneal_bipartite(tb, 1, lv0.copy(), rv0.copy(), Jb, lb, rb,
                                                        np.random.RandomState(4)))))
    rows_out = []
    for name, updates, make in cases:
        mod_ours = d_sa if name.startswith("sa.") else d_qmc
        call = make(mod_ours)
        call()                                     # warm-up: kernel load, first-call set-up
        ours = min(timed(call) for _ in range(2))
        row = {"call": name, "updates": updates, "ours_s": ours, "ours_updates_per_s": updates / ours}
        if ref is not None:
            rcall = make(ref[1] if name.startswith("sa.") else ref[0])
            rs = timed(rcall)
            row.update(reference_s=rs, reference_updates_per_s=updates / rs, speedup_vs_one_core=rs / ours)
        rows_out.append(row)
    out["calls"] = rows_out
    return out


def generators_workload(args, torch):
    """Instance generation: the GPU table generator against the host drop-in generator + GenerateNeighbors."""
    from piqmc import tools
    out = {"note": "GPU: tools.lattice_table (neighbour table written in device memory, CUDA events); host: the "
                   "drop-in generator (the caller's MT19937 values, as the reference) + GenerateNeighbors, wall time"}
    cases = [("ising2d 80x80 torus", "ising2d", 80, 80, 1, lambda: tools.Generate2DIsingInstance(
                 80, np.random.RandomState(0)), 4),
             ("kblock 64x64 k=2", "kblock", 64, 64, 2, lambda: tools.GenerateKblockLattice(
                 64, 64, np.random.RandomState(0), k=2), 24)]
    rows = []
    for name, kind, r, c, k, host, maxnb in cases:
        tools.lattice_table(kind, r, c, seed=1, k=k, maxnb=maxnb)            # warm-up
        ms = []
        for _ in range(3):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            tools.lattice_table(kind, r, c, seed=1, k=k, maxnb=maxnb, check=False)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        t0 = time.perf_counter()
        J = host()
        tools.GenerateNeighbors(r * c, J, maxnb)
        host_ms = (time.perf_counter() - t0) * 1e3
        rows.append({"instance": name, "gpu_ms": min(ms), "host_ms": host_ms, "speedup": host_ms / min(ms)})
    out["instances"] = rows
    return out


def only_arm(args):
    """One extra workload on its own (profiling entry point)."""
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    args.no_cpu_baseline = True
    if args.only == "batched":
        out = batched_workload(args, torch)
    elif args.only == "dense":
        out = dense_workload(args, torch)
    elif args.only == "reforder":
        out = reforder_workload(args, torch)
    elif args.only == "gemm":
        out = gemm_workload(args, torch)
    elif args.only == "dropin":
        out = dropin_workload(args, torch)
    elif args.only == "generators":
        out = generators_workload(args, torch)
    else:
        from piqmc import fast, tools
        import scipy.sparse as sps
        n = L_SIDE * L_SIDE
        rows, cols, vals = instance_arrays()
        J = sps.dok_matrix((n, n))
        for a, b, v in zip(rows, cols, vals):
            J[int(a), int(b)] = v
        out = learned_vs_plain(args, torch, fast.Problem(tools.GenerateNeighbors(n, J, 4)), R=args.learned_replicas)
    print(json.dumps({"only": args.only, **out}, default=float), flush=True)


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    base = cpu_baseline(steps=args.steps, warmup=args.warmup)
    # n_gpus mirrors the GPU arm's launch; the work itself runs on the host cores (cpu_baseline.cores)
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": "updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32/fp64", "data": "synthetic",
            "config": {"workload": "80x80 periodic lattice, J~N(0,1) fp32, P=20, T=0.05, G linear 3.0->1e-8; "
                                   "each step a bounded sample of the 2000-step schedule: every 20th field value "
                                   "(100 steps, 1.28e7 updates per process), one replica per host core",
                       "sample": base["sample"],
                       "parallelism": "%d host processes" % base["cores"]},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--replicas", type=int, default=REPLICAS)
    ap.add_argument("--nsched", type=int, default=NSCHED)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--rpc", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched, dense and learned extras")
    ap.add_argument("--only", choices=["batched", "dense", "learned", "reforder", "gemm", "dropin", "generators"], default=None,
                    help="run one extra workload alone (for profiling) and print its JSON")
    ap.add_argument("--batched-count", type=int, default=256)
    ap.add_argument("--batched-steps", type=int, default=500)
    ap.add_argument("--dense-replicas", type=int, default=256)
    ap.add_argument("--dense-steps", type=int, default=1000)
    ap.add_argument("--learned-replicas", type=int, default=1024)
    ap.add_argument("--reforder-steps", type=int, default=100)
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    elif args.only:
        only_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()

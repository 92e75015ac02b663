#!/usr/bin/env python3
"""bench.py — throughput of the GB300 force/energy hot path.

Workload: the polyelectrolyte solution (64 chains x 200 beads, 12800
counterions, 20000 salt pairs; N = 65600 ions, L = 700 A, SPME order 6 on a
128^3 mesh, r_c = 12 A, Verlet skin 2 A), overdamped BD (BDStep + UTotal +
list check per step, dt = 0.01 ps).  A step is one BD step of the whole
system.  Inputs are seeded synthetic configurations (no dataset exists).

Timing: W untimed warm-up steps, then K device steps; before every step an
untimed write of 512 MiB evicts the L2 cache (the system fits in L2, so it is
flushed rather than outgrown), and an untimed read of the same buffer has
the write's dirty lines written back before the step starts; CUDA events on
the library's stream bracket
each step; the per-step times are summed.  `value` is the mixed form
(FP32 arithmetic, 64-bit fixed-point accumulation); the plain FP64 form is
reported beside it.  `e2e` runs the same steps through the C ABI with host
buffers (positions in, positions and forces out every step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --impl reference the CPU oracle (the C restatement of the reference's
Fortran) runs BD steps of the same workload on every host core, its threads
standing in for the reference's MPI ranks (replicated data, particle ranges
per rank); each step is timed on the host.  The default run also reports the
oracle on one thread, the reference's serial build (molsim_ser).

Accuracy: the oracle's FP64 UTotal of the same configuration is the
reference for the force and energy errors of both GPU forms.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MD steps/s @65k-ion SPME: mixed vs FP64 GPU at force RMS≤1e-5; host-CPU ref"
FLUSH_BYTES = 512 << 20
BD_DT = 0.01
BD_SEED = 1234567
WORKLOAD = "polyelectrolyte N=65600 (64x200 beads, 12800 counterions, 20000 salt pairs) L=700A SPME p=6 128^3 r_c=12A BD"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def replica_seed(seed, rank):
    """Replicas only: every rank runs its own independent system."""
    return seed + rank


def barrier(world):
    """All ranks reach this point, then the local device is idle."""
    import torch
    if world > 1:
        torch.distributed.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def max_over_ranks(x, world, device="cuda"):
    """Max of a per-rank float over all ranks (the slowest rank sets the time)."""
    if world == 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def make_system(seed):
    from molsim_gb300 import configs
    t = time.time()
    s = configs.polyelectrolyte(seed=seed)
    log(f"[bench] workload generated in {time.time() - t:.1f}s (N={s.np_})")
    return s


# ---- algorithmic bytes per launch of each phase (mixed form) -------------------
# Each logical array counts once per launch at the form's element size: N
# particles, P stored neighbour pairs, K the mesh edge, p the spline order, nb
# bonds.  Positions 24 B (FP64 xyz), charges 8 B, fixed-point forces 24 B (read
# and written where they accumulate), spline values 4 B, the real mesh 4 B and
# the half spectrum 8 B per point.  Tile halos, re-reads and atomics are not
# algorithmic and are not counted.
def algorithmic_bytes(kernel, n, k, pairs, nbond, order=6):
    nh = k // 2 + 1
    k3, spec = k ** 3, nh * k * k
    spl = 3 * order * 4                       # one set of spline values per particle
    return {
        "bd_rng": n * 12,                                     # 3 deviates out
        "bd_move": n * (24 + 24 + 12 + 24),                   # ro, force, deviates in; ro out
        "list": n * 24,                                       # displacement check
        "prepare": n * (24 + 4 + 16),                         # ro, type in; cell slot out
        "pair": n * 16 + pairs * 4 + n * 48,                  # slots, list in; forces in+out
        "splines": n * 24 + n * (12 + 2 * spl),               # ro in; corner, w, dw out
        "brick_sort": n * (12 + 12),                          # corner in; brick, rank, perm out
        "spread": n * (4 + 12 + spl + 8) + k3 * 4,            # perm, corner, w, q in; mesh out
        # plane sort: plane and rank in, the spread record (corner, charge,
        # z/x/y values) in and out
        "plane_sort": n * (4 + 4) + 2 * n * (8 + spl),
        # spread inside the forward plane pass: spread records in; half spectrum out
        "spread+fft_xy": n * (8 + spl) + spec * 8,
        "mesh_fold": k3 * 4,                                  # mesh out
        "fft_x_r2c": k3 * 4 + spec * 8,
        "fft_y_fwd": 2 * spec * 8,
        "fft_z_conv": 2 * spec * 8 + 3 * nh ** 3 * 4,         # spectrum in+out, influence tables
        "fft_y_inv": 2 * spec * 8,
        "fft_x_c2r": spec * 8 + k3 * 4,
        "fft_xy_fwd": k3 * 8 * 2 + spec * 8,                  # fixed-point mesh in and cleared; spectrum out
        "fft_yx_inv": spec * 8 + k3 * 4,                      # spectrum in; potential mesh out
        "gather": k3 * 4 + n * (4 + 12 + 2 * spl + 8) + n * 48,
        "bond+reduce": nbond * 48 + n * 48,
    }.get(kernel)


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        import threading
        self.lines = []
        self.first = threading.Event()
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self

        def reader():
            for line in self.proc.stdout:
                self.lines.append(line)
                self.first.set()
        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()
        # the timed region starts once the sampler runs (nvidia-smi takes
        # about a second to start)
        self.first.wait(timeout=10.0)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=5)
        self.out = "".join(self.lines)
        return False

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def utotal_errors(g, r):
    """Errors of a GPU UTotal against the oracle's: RMS and largest
    per-particle force error over the RMS force, energy and virial relative
    errors."""
    d = np.asarray(g["forceo"]).reshape(-1, 3) - np.asarray(r["forceo"]).reshape(-1, 3)
    fr = np.asarray(r["forceo"]).reshape(-1, 3)
    frms = float(np.sqrt((fr * fr).sum(1).mean()))
    dn = np.sqrt((d * d).sum(1))
    return {"force_rms": float(np.sqrt((dn * dn).mean()) / frms), "force_max": float(dn.max() / frms),
            "energy_rel": abs(g["u_tot"] - r["u_tot"]) / abs(r["u_tot"]),
            "u_rec_rel": abs(g["u_rec"] - r["u_rec"]) / abs(r["u_rec"]),
            "virial_rel": abs(g["virial"] - r["virial"]) / abs(r["virial"])}


def cpu_threads():
    """Host threads for the CPU reference: every core this process may use."""
    try:
        n = len(os.sched_getaffinity(0))
    except AttributeError:
        n = os.cpu_count() or 1
    return max(1, min(64, n))


def cpu_baseline(seed, budget_s=20.0, max_steps=12, warmup=1, threads=1, initial=None):
    """The oracle on BD steps of the same workload, with `threads` threads
    standing in for the reference's MPI ranks (replicated data, particle
    ranges per rank, partial sums combined in rank order); cell-list mode so
    that set-up is O(N) (the Verlet-list build is O(N^2)).  Returns the host
    time of each step; with `initial` (a dict), also the oracle's FP64 UTotal
    of the initial configuration (forces, energies, virial) in it, the
    reference for the GPU forms' errors."""
    from molsim_gb300 import Engine, abi
    from oracle.loader import oracle
    orc = oracle()
    if orc.orc_set_threads(threads) != 0:
        raise RuntimeError(f"oracle: {threads} threads refused")
    try:
        s = make_system(seed)
        s.txintlist = abi.MG_CELLLIST
        s.build_table(orc.orc_pot_twobody_tab)
        e = Engine(s, lib=orc, prefix="orc_")
        e.SetPositions(s.ro_flat())
        e.NList("write")
        e.BDSetup(BD_DT, BD_SEED)
        r0 = e.BDRun(0)  # initial forces, untimed
        if initial is not None:
            initial.update(r0)
        for _ in range(warmup):
            e.BDRun(1)
        times = []
        t_all = time.perf_counter()
        while len(times) < max_steps and time.perf_counter() - t_all < budget_s:
            t0 = time.perf_counter()
            e.BDRun(1)
            times.append(time.perf_counter() - t0)
        e.close()
    finally:
        orc.orc_set_threads(1)
    return times


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return 0
    nt = cpu_threads()
    times = cpu_baseline(args.seed, budget_s=min(60.0, 2.0 * max(args.steps, 1)), max_steps=max(args.steps, 1),
                         warmup=args.warmup, threads=nt)
    v = len(times) / sum(times)
    sample = (f"{len(times)} BD steps of the full N=65600 workload (oracle, cell-list mode, {nt} threads as "
              "the reference's MPI ranks), host wall clock per step")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": len(times), "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "form": f"reference CPU FP64 (oracle port, {nt} threads)"},
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": nt, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)
    return 0


def run_ours(args):
    import torch

    import molsim_gb300
    from molsim_gb300 import Engine, abi

    rank, local_rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev_index = torch.cuda.current_device()
    molsim_gb300.build()
    s = make_system(replica_seed(args.seed, rank))
    s.build_table()
    K, W = args.steps, args.warmup

    def engine(form):
        e = Engine(s, form=form)
        e.SetPositions(s.ro_flat())
        e.NList("write")
        e.BDSetup(BD_DT, BD_SEED)
        return e

    # UTotal of the initial configuration in both forms; their errors against
    # the oracle's FP64 UTotal of the same configuration come with the CPU
    # baseline below
    e64, emx = engine(abi.MG_FP64), engine(abi.MG_MIXED)
    r64, rmx = e64.UTotal(), emx.UTotal()

    results = {}
    clocks = None
    for name, e in (("fp64", e64), ("mixed", emx)):
        e.BenchSteps(1, W, FLUSH_BYTES)
        barrier(world)
        calls0 = e.NListCalls()
        if name == "mixed":
            with ClockSampler(dev_index) as cs:
                ms = e.BenchSteps(1, K, FLUSH_BYTES)
            clocks = cs.summary()
        else:
            ms = e.BenchSteps(1, K, FLUSH_BYTES)
        barrier(world)
        ms = max_over_ranks(ms, world)
        results[name] = {"ms_per_step": ms / K, "steps_per_s": world * K / (ms * 1e-3),
                         "list_rebuilds": e.NListCalls() - calls0}
    kernels_per_step = emx.StepKernels(1)

    # per-kernel device times (uncaptured launches, same flush regime)
    def phase_pass(e):
        e.PhaseReset(True)
        e.BenchSteps(1, min(50, max(K, 5)), FLUSH_BYTES)
        ph = e.PhaseTimes()
        e.PhaseReset(False)
        return ph
    phases = phase_pass(emx)
    phases64 = phase_pass(e64)
    nn, _ = emx.VList(maxnneigh=256)
    pairs = int(2 * nn.sum())
    nbond = 0 if s.bond_ip is None else len(s.bond_ip)
    # the Verlet-list rebuild runs on a small fraction of the steps; its
    # per-call time is reported but does not pick the dominant kernel
    dom = max((k for k in phases if k != "list_build"), key=phases.get)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_src = 6800.0, "fallback"
    ab = algorithmic_bytes(dom, s.np_, s.nmesh, pairs, nbond, s.order)
    achieved = ab / (phases[dom] * 1e-3) / 1e9 if ab else None

    # end to end through the C ABI with host buffers
    lib = abi.load_library()
    n3 = 3 * s.np_
    ro_h = torch.empty(n3, dtype=torch.float64, pin_memory=True)
    f_h = torch.empty(n3, dtype=torch.float64, pin_memory=True)
    u_h = torch.empty(4, dtype=torch.float64, pin_memory=True)
    ro_h.copy_(torch.from_numpy(emx.GetPositions().reshape(-1)))
    p_ro = C.cast(ro_h.data_ptr(), abi.PF64)
    p_f = C.cast(f_h.data_ptr(), abi.PF64)
    p_u = C.cast(u_h.data_ptr(), abi.PF64)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    ke = max(1, min(K, 500))
    for _ in range(min(W, 10)):
        assert lib.mg_bd_step_host(emx.h, p_ro, p_f, p_u) == 0
    tsum = 0.0
    barrier(world)
    for i in range(ke):
        flush.fill_(float(i))
        flush.sum()   # the written lines read back: clean before the step
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = lib.mg_bd_step_host(emx.h, p_ro, p_f, p_u)
        tsum += time.perf_counter() - t0
        if st != 0:
            raise RuntimeError(f"mg_bd_step_host failed: {st}")
    tsum = max_over_ranks(tsum, world)
    e2e = world * ke / tsum

    cpu = cpu1 = None
    accuracy = {"reference": "none (--no-cpu)"}
    if rank == 0 and not args.no_cpu:
        nt = cpu_threads()
        ref0 = {}
        times = cpu_baseline(args.seed, threads=nt, initial=ref0)
        cpu = {"value": len(times) / sum(times), "unit": "steps/s", "cores": nt, "kind": "port",
               "sample": f"{len(times)} BD steps of the full N=65600 workload on {nt} host threads "
                         "(oracle, cell-list mode, threads as the reference's MPI ranks), wall clock per step"}
        times1 = cpu_baseline(args.seed, budget_s=10.0, max_steps=5, warmup=0, threads=1)
        cpu1 = {"value": len(times1) / sum(times1), "unit": "steps/s", "cores": 1, "kind": "port",
                "sample": f"{len(times1)} BD steps of the full N=65600 workload on one host thread "
                          "(oracle, cell-list mode: the reference's serial build), wall clock per step"}
        accuracy = {"reference": "oracle FP64 UTotal of the same configuration (CPU restatement of the "
                                 "reference), forces per particle",
                    "mixed": utotal_errors(rmx, ref0), "fp64": utotal_errors(r64, ref0),
                    "bar": {"force_rms": 1e-5}}

    if rank == 0:
        out = {
            "metric": METRIC, "value": results["mixed"]["steps_per_s"], "unit": "steps/s",
            "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": results["mixed"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64",
            "data": "synthetic (seeded polyelectrolyte configuration)",
            "config": {"workload": WORKLOAD, "form": "mixed (FP32 arithmetic, int64 fixed-point accumulation)",
                       "l2": "flushed before every timed step (512 MiB written, then read back so its dirty lines are written back outside the timed step)",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "fp64": results["fp64"],
            "mixed_over_fp64": results["mixed"]["steps_per_s"] / results["fp64"]["steps_per_s"],
            "list_rebuilds": {"mixed": results["mixed"]["list_rebuilds"],
                              "fp64": results["fp64"]["list_rebuilds"], "steps": K},
            "accuracy": accuracy,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_source": peak_src, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": None,
                         "algorithmic_bytes": ab, "kernel_ms": phases[dom]},
            "phases_ms": phases,
            "phases_ms_fp64": phases64,
            "cpu_baseline": cpu,
            "cpu_baseline_1thread": cpu1,
            "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": 24 * s.np_,
                    "d2h_bytes_per_step": 48 * s.np_ + 32},
            "clocks": clocks,
            "gpu_launches": kernels_per_step * K,
        }
        print(json.dumps(out), flush=True)
    for e in (e64, emx):
        e.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_profile(args):
    """A short, quiet run for ncu: the workload in one form, W warm-up steps
    and K steps through the captured step graph, no flush, no other work."""
    import torch

    import molsim_gb300
    from molsim_gb300 import Engine, abi
    torch.cuda.set_device(0)
    molsim_gb300.build()
    s = make_system(args.seed)
    s.build_table()
    e = Engine(s, form=abi.MG_MIXED if args.profile == "mixed" else abi.MG_FP64)
    e.SetPositions(s.ro_flat())
    e.NList("write")
    e.BDSetup(BD_DT, BD_SEED)
    # phase timing runs the steps as plain launches: ncu does not profile the
    # kernels of a graph that holds a conditional node
    e.PhaseReset(True)
    ms = e.BenchSteps(1, args.warmup + args.steps, 0)
    log(f"[profile] {args.profile}: {args.warmup + args.steps} steps, {ms:.3f} ms, "
        f"{e.StepKernels(1)} kernels per step")
    e.close()
    return 0


def run_water(args):
    """The polyatomic path on its own (not the headline workload): UTotal of
    rigid three-site waters and ions with SPME over the atom charges
    (PolyEngine.UTotal: the atom-pair loop, the atoms' reciprocal sum, the
    molecular self term, particle forces and torques), host arrays in and
    out every call as the reference's argument-less routines see them; the
    atom-pair loop alone; and rigid-body MD steps of the same particles,
    host-driven (PolyEngine.VelVer) and on the device (mg_poly_md_run).  One
    JSON line, rank 0."""
    import torch

    import molsim_gb300
    from molsim_gb300 import abi, configs
    from molsim_gb300.poly import PolyEngine
    torch.cuda.set_device(0)
    molsim_gb300.build()
    t = time.time()
    s = configs.water_ions(seed=args.seed, nwater=4000, nsalt=100, L=58.0, rcut=10.0)
    s.relpermitt = 78.0
    s.ewald, s.ualpha, s.order, s.nmesh = abi.MG_EWALD_SPM, 0.35, 6, 64
    s.build_table(abi.load_library().mg_pot_twobody_tab)
    L = s.boxlen[0]
    d = s.ro[:, None, :] - s.ro[None, :, :]
    d -= L * np.round(d / L)
    near = ((d * d).sum(-1) <= (s.rcut + 1.0) ** 2) & np.triu(np.ones((s.np_, s.np_), dtype=bool), 1)
    nn = near.sum(1).astype(np.int32)
    maxn = int(nn.max())
    jl = np.zeros((s.np_, maxn), dtype=np.int32)
    for i in range(s.np_):
        js = np.flatnonzero(near[i]) + 1
        jl[i, :len(js)] = js
    log(f"[bench] water workload generated in {time.time() - t:.1f}s (particles {s.np_}, atoms {len(s.iatan())})")
    e = PolyEngine(s, maxn)
    for _ in range(args.warmup):
        e.UTotal(nn, jl)
        e.UTotal()
    K = max(1, min(args.steps, 200))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        out = e.UTotal(nn, jl)
    t_tot = (time.perf_counter() - t0) / K
    t0 = time.perf_counter()
    for _ in range(K):
        e.UTwoBodyP(nn, jl)
    t_pair = (time.perf_counter() - t0) / K
    t0 = time.perf_counter()
    for _ in range(K):
        out_dev = e.UTotal()
    t_tot_dev = (time.perf_counter() - t0) / K
    t0 = time.perf_counter()
    for _ in range(K):
        e.UTwoBodyPList()
    t_pair_dev = (time.perf_counter() - t0) / K
    # rigid-body MD (VelVer with quaternions) of the same particles: the
    # host between the parts of every step, then every step on the device
    r = s.principal_axes()
    r.build_table(abi.load_library().mg_pot_twobody_tab)
    rng = np.random.default_rng(args.seed)
    massip, momp = r.rigid_props()
    kt = 8.314472e-3 * 298.0
    v = rng.standard_normal((r.np_, 3)) * np.sqrt(kt * massip / 0.01)[:, None]
    w = np.where(momp > 0.0, rng.standard_normal(momp.shape) * np.sqrt(kt / (0.01 * np.maximum(momp, 1e-300))), 0.0)
    em = PolyEngine(r, maxn)
    em.RigidSetup(0.0005, v, w, prime=True)
    Km = max(1, min(args.steps, 50))
    em.VelVer(2)
    t0 = time.perf_counter()
    em.VelVer(Km)
    t_md_host = (time.perf_counter() - t0) / Km
    em.MDRun(2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    md = em.MDRun(Km)
    t_md_dev = (time.perf_counter() - t0) / Km
    em.close()
    print(json.dumps({
        "metric": "polyatomic UTotal calls/s (rigid waters and ions, SPME over atoms), host arrays each call",
        "value": 1.0 / t_tot, "unit": "calls/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_call": 1e3 * t_tot, "ms_atom_pair_loop": 1e3 * t_pair,
        "device_list": {"ms_per_call": 1e3 * t_tot_dev, "ms_atom_pair_loop": 1e3 * t_pair_dev,
                        "u_tot": out_dev["u_tot"]},
        "rigid_md": {"steps": Km, "dt_ps": 0.0005, "host_driven_ms_per_step": 1e3 * t_md_host,
                     "device_ms_per_step": 1e3 * t_md_dev, "device_steps_per_s": 1.0 / t_md_dev,
                     "u_tot": md["u_tot"]},
        "higher_is_better": True,
        "dtype": "f64", "data": "synthetic (seeded rigid waters and NaCl)",
        "config": {"workload": f"{s.np_} particles, {len(s.iatan())} atoms, L={L} A, r_c={s.rcut} A, "
                               f"SPME p={s.order} {s.nmesh}^3", "u_tot": out["u_tot"]}}))
    e.close()
    return 0


def run_replicas(args):
    """The batched configuration (not the headline workload): nrep
    independent electrolyte boxes, N log-uniform in [500, 8000], salt
    uniform in [0.01, 1.0] M, charges +-1 e, LJ sigma = 4 A, eps = 0.1 kT;
    SPME order 6 with the real-space cutoff and mesh chosen per box for a
    force RMS error of 1e-5 (autotune.choose_spme).  Timed: K MD steps of
    all boxes (mixed form, one CUDA graph launch per step over every box),
    then 10^4 single-ion displacement trials (dtran = 2 A) per box through
    the denergy path (mg_dutotal_batch, FP64).  Reported: aggregate box-steps
    per second, trials per second, every box's mixed-form force RMS error
    against its FP64 form, and the SPME error against a converged FP64
    reference measured on a sample of boxes.  One JSON line, rank 0."""
    import dataclasses

    import torch

    import molsim_gb300
    from molsim_gb300 import Engine, abi, autotune, configs
    from molsim_gb300.ensemble import Ensemble
    torch.cuda.set_device(0)
    molsim_gb300.build()
    nrep = args.replicas
    t = time.time()
    rs = configs.replica_set(seed=args.seed, nrep=nrep, mode=abi.MG_MD)
    conc, choice = [], []
    for s in rs:
        c = (s.np_ / 2) / (float(np.prod(s.boxlen)) * 1e-27 * configs.AVOGADRO)
        ch = autotune.choose_spme(s, c, ns_per_point=args.mesh_ns)
        s.rcut, s.ualpha, s.order, s.nmesh = ch["rcut"], ch["ualpha"], ch["order"], ch["nmesh"]
        s.build_table()
        conc.append(c)
        choice.append(ch)
    log(f"[bench] {nrep} replicas generated and tabulated in {time.time() - t:.1f}s "
        f"({sum(s.np_ for s in rs)} ions)")

    def engine(s, form, mode=abi.MG_MD):
        e = Engine(dataclasses.replace(s, mode=mode), form=form)
        e.SetPositions(s.ro_flat())
        e.NList("write")
        return e

    # per box: the mixed form against the FP64 form of the same settings
    err_mixed = []
    for s in rs:
        e64, emx = engine(s, abi.MG_FP64), engine(s, abi.MG_MIXED)
        f64, fmx = e64.UTotal()["forceo"], emx.UTotal()["forceo"]
        e64.close()
        emx.close()
        err_mixed.append(float(np.sqrt(((fmx - f64) ** 2).mean() / (f64 ** 2).mean())))
    # the SPME setting against a converged FP64 reference (order 10, twice
    # the mesh up to 256) on boxes spread over the concentrations
    order_c = np.argsort(conc)
    sample = sorted(set(int(order_c[int(i)]) for i in np.linspace(0, nrep - 1, min(8, nrep))))
    err_spme = []
    for i in sample:
        s = rs[i]
        ref = dataclasses.replace(s, order=10, nmesh=min(256, 2 * s.nmesh))
        er, e0 = engine(ref, abi.MG_FP64), engine(s, abi.MG_FP64)
        fr, f0 = er.UTotal()["forceo"], e0.UTotal()["forceo"]
        er.close()
        e0.close()
        err_spme.append({"box": i, "N": s.np_, "c_M": round(conc[i], 4), "rcut": s.rcut, "nmesh": s.nmesh,
                         "ref_nmesh": ref.nmesh,
                         "force_rms": float(np.sqrt(((f0 - fr) ** 2).mean() / (fr ** 2).mean()))})

    # MD: all boxes, one graph launch per step
    engines = []
    for i, s in enumerate(rs):
        e = engine(s, abi.MG_MIXED)
        e.MDSetup(0.002, s.maxwell_velocities(seed=1000 + i))
        engines.append(e)
    ens = Ensemble(engines)
    K, W = args.steps, args.warmup
    ens.run(0, W)
    torch.cuda.synchronize()
    with ClockSampler(0) as cs:
        ms = ens.run(0, K)
    clocks = cs.summary()
    kernels = ens.kernels(0)
    ens.close()
    for e in engines:
        e.close()

    # MC: 10^4 single-ion trials per box, FP64 denergy path
    ntrial = args.trials
    rng = np.random.Generator(np.random.PCG64(args.seed))
    t_mc = 0.0
    for s in (rs if ntrial > 0 else []):
        e = engine(s, abi.MG_FP64, abi.MG_MC)
        e.UTotal()
        ip = rng.integers(1, s.np_ + 1, ntrial).astype(np.int32)
        ro = s.ro[ip - 1] + 2.0 * (rng.random((ntrial, 3)) - 0.5)
        ro -= s.boxlen * np.round(ro / s.boxlen)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        du, ovl = e.DUTotalBatch(ip, ro)
        t_mc += time.perf_counter() - t0
        e.close()
    box_steps = nrep * K / (ms * 1e-3)
    print(json.dumps({
        "metric": "batched replicas: box MD steps/s (mixed) and MC trial dU/s (FP64)",
        "value": box_steps, "unit": "box-steps/s", "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "dtype": "f32+i64",
        "data": "synthetic (seeded replica set)",
        "config": {"workload": f"{nrep} electrolyte boxes, N log-uniform in [500, 8000], c uniform in [0.01, 1.0] M, "
                               "SPME order 6, r_c and mesh per box for force RMS 1e-5",
                   "ions": int(sum(s.np_ for s in rs)),
                   "settings": {f"rc{int(k[0])}_K{k[1]}": v for k, v in sorted(
                       __import__("collections").Counter((s.rcut, s.nmesh) for s in rs).items())},
                   "l2": "not flushed: the boxes' meshes and particles together exceed the 129 MB L2"},
        "ensemble_steps_per_s": K / (ms * 1e-3),
        "mc": {"trials_per_box": ntrial, "trials_per_s": nrep * ntrial / t_mc if t_mc > 0 else None,
               "note": "host wall clock of mg_dutotal_batch per box (copies in and out included)"},
        "accuracy": {"mixed_vs_fp64_force_rms": {"max": max(err_mixed), "median": float(np.median(err_mixed))},
                     "spme_vs_converged_sample": err_spme},
        "kernels_per_step": kernels, "clocks": clocks,
    }), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--profile", choices=["mixed", "fp64"],
                    help="profiling run for ncu: only W + K BD steps of one form, nothing else")
    ap.add_argument("--workload", choices=["polyelectrolyte", "water", "replicas"], default="polyelectrolyte",
                    help="water: the polyatomic path on its own; replicas: the batched boxes (not the headline metric)")
    ap.add_argument("--replicas", type=int, default=256, help="boxes of the replicas workload")
    ap.add_argument("--trials", type=int, default=10000, help="MC trials per box of the replicas workload")
    ap.add_argument("--mesh-ns", type=float, default=0.01,
                    help="replicas workload: modelled ns per mesh point when choosing r_c and the mesh")
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.workload == "water":
        return run_water(args)
    if args.workload == "replicas":
        return run_replicas(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

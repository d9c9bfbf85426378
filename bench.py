"""Benchmark: wall time of one full Newton time step of the lithosphere model
(1025 x 513 grid over 1000 x 400 km, 4 phases, 16 markers per cell ~ 8.4 M
markers) on one GB300, in the plain FP64 form and in the FP32-refined
(+ learned local-rheology guess, when an MLP is loaded) form.

A step is one pass of the hot path: marker->grid projection, the Newton loop
to a 1e-8 relative Stokes residual (local VEP rheology + tangent, matrix-free
residual / Jacobian, GCR + multigrid, line search), marker stress/strain
update and RK4 advection.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  For N > 1 (torchrun) every rank runs an
independent replica of the model (the build does not shard the path).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "mdoodz6.0_gb300"), os.path.join(ROOT, "oracle")]

METRIC = "Newton-step time @1025x513: learned+FP32-IR vs plain FP64 GPU, 1e-8 resid"
UNIT = "ms/step"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([s.strip() for s in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        import statistics
        mhz = [float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for nm, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return d["hbm_gbs"], d.get("bf16_tflops"), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


# the local-rheology MLP workload: 2^24 tuples over these ranges, batch 65536
LO_MLP, HI_MLP = [-18.0, 273.0, 0.0, 9.0], [-12.0, 1600.0, 5e9, 12.0]


GUESS_STEPS = [3000]

# DRAM bytes (read + write) per launch of a kernel class at 1025x513, from one
# ncu capture of the FP32 form (dram__bytes_read.sum + dram__bytes_write.sum
# over the kernels of 8 preconditioner applications, caches left warm)
TRAFFIC_PER_LAUNCH = {"mg_vcycle": 88.5e6}


def train_guess(ctx, cfg):
    """The learned start of the model (mdz_setups.train_guess); returns
    (seconds, final loss)."""
    import mdz_setups
    t0 = time.perf_counter()
    loss = mdz_setups.train_guess(ctx, cfg, steps=GUESS_STEPS[0])
    return time.perf_counter() - t0, loss


def run_form(cfg_builder, precision, learned, steps, warmup, size, reseed=False):
    import numpy as np
    import mdz
    import mdz_setups
    cfg = cfg_builder(precision, learned, size)
    g = cfg["grid"]
    ctx = mdz_setups.load_context(cfg, max_markers=marker_capacity(cfg))
    model, mat = cfg["model"], cfg["mat"]
    train = train_guess(ctx, cfg) if learned else None
    reps = []
    for _ in range(warmup):
        ctx.time_step(mat, model)
    ctx.L.mdz_sync(ctx.h)
    ctx.set_profiling(True)
    l0 = ctx.kernel_launches
    t0 = time.perf_counter()
    marks = []
    for _ in range(steps):
        reps.append(ctx.time_step(mat, model).as_dict())   # synchronous: returns when the step is done
        marks.append(time.perf_counter())
    ctx.L.mdz_sync(ctx.h)
    wall = (time.perf_counter() - t0) * 1e3 / steps
    step_ms = [(b - a) * 1e3 for a, b in zip([t0] + marks[:-1], marks)]
    launches = ctx.kernel_launches - l0
    gpu_ms = sum(r["ms_total"] for r in reps) / steps
    kern = ctx.kernel_timing()
    g = cfg["grid"]
    final = {"u": np.empty(g.size(-1)), "v": np.empty(g.size(-2)), "p": np.empty(g.size(1))}
    ctx._check(ctx.L.mdz_get_velocity(ctx.h, mdz._dptr(final["u"]), mdz._dptr(final["v"]), mdz._dptr(final["p"])))
    final["sxxd"] = ctx.get_marker_attr(mdz.M_SXXD)
    final["sxz"] = ctx.get_marker_attr(mdz.M_SXZ)
    n_final = ctx.n_markers
    ctx.close()
    rs = reseed_pass(cfg) if reseed else None
    return dict(ms_wall=wall, ms_gpu=gpu_ms, reports=reps, launches=launches, kernel=kern, cfg=cfg, train=train,
                final=final, reseed=rs, step_ms=step_ms, n_markers_final=n_final)


def marker_capacity(cfg):
    import mdz_setups
    return mdz_setups.marker_capacity(cfg)


def reseed_pass(cfg, min_part_cell=16):
    """One reseeding pass (CountPartCell with RESEED = 1, DirectNeighbour = 1)
    of the configuration's seeded markers, through the C ABI: wall time of the
    synchronous call (a pass with min_part_cell = 0, which adds nothing, sets
    up its workspace first).  The CPU side is the oracle's one-thread
    restatement on the same markers."""
    import mdz
    import mdz_setups
    import oracle
    ctx = mdz_setups.load_context(cfg, max_markers=marker_capacity(cfg))
    x, z, ph, vx, vz = ctx.get_markers()
    m = dict(x=x, z=z, phase=ph, vx=vx, vz=vz)
    for k, a in zip(oracle.MARKER_ATTRS, range(mdz.M_NATTR)):
        m[k] = ctx.get_marker_attr(a)
    n = len(x)
    ctx.CountPartCell(1, 0, 1)
    ctx.L.mdz_sync(ctx.h)
    t0 = time.perf_counter()
    added = ctx.CountPartCell(1, min_part_cell, 1)
    ms = (time.perf_counter() - t0) * 1e3
    ctx.close()
    g = cfg["grid"]
    t0 = time.perf_counter()
    _, added_cpu = oracle.reseed(g, m, marker_capacity(cfg), min_part_cell, 1)
    ms_cpu = (time.perf_counter() - t0) * 1e3
    # algorithmic bytes: marker x, z, phase read twice (bins, candidates), one
    # int bin index written and read, quarter-cell counts, and the new markers
    # written with their 12 copied values
    nq = (2 * g.ncx + 4) * (2 * g.ncz + 4)
    byts = n * (2 * 20 + 8) + nq * 16 + added * (12 * 8 + 16)
    return {"markers": n, "added": added, "ms": ms, "GB/s": byts / (ms * 1e-3) / 1e9,
            "cpu_baseline": {"value": ms_cpu, "unit": "ms", "cores": 1, "kind": "port", "added": added_cpu,
                             "sample": "the same markers, one pass"}}


def field_diffs(a, b):
    import numpy as np
    out = {}
    for k in a:
        x, y = a[k], b[k]
        if k == "p":
            x, y = x - x.mean(), y - y.mean()
        out[k] = float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))
    return out


PARITY_GRID = (129, 65)


def parity_vs_oracle(nx=PARITY_GRID[0], nz=PARITY_GRID[1]):
    """Each output field of both GPU forms after one time step of the
    lithosphere model at nx x nz, against the oracle's FP64 time step on the
    same inputs (restated reference functions, exact defect solves): relative
    2-norm errors (pressure with its mean removed: the operator leaves it
    undetermined)."""
    import numpy as np
    import mdz
    import mdz_setups
    import oracle_step
    cfg = mdz_setups.config_lithosphere(Nx=nx, Nz=nz, precision=64)
    m = {k: v.copy() for k, v in cfg["markers"].items()}
    u, v, p, rep = oracle_step.time_step(cfg["grid"], cfg["mat"], cfg["model"], m, cfg["u"], cfg["v"], cfg["p"])
    ref = dict(u=u, v=v, p=p - p.mean(), sxxd=m["sxxd"], szzd=m["szzd"], sxz=m["sxz"], x=m["x"], z=m["z"])
    out = {"grid": "%dx%d" % (nx, nz), "step": 1, "oracle_nonlinear_its": rep["nonlinear_its"]}
    for name, prec, learned in (("plain_fp64", 64, 0), ("learned_fp32_ir", 32, 1)):
        c = mdz_setups.config_lithosphere(Nx=nx, Nz=nz, precision=prec, learned=learned)
        ctx = mdz_setups.load_context(c)
        if learned:
            mdz_setups.train_guess(ctx, c, steps=GUESS_STEPS[0])
        r = ctx.time_step(c["mat"], c["model"])
        g = c["grid"]
        uu, vv, pp = np.empty(g.size(-1)), np.empty(g.size(-2)), np.empty(g.size(1))
        ctx._check(ctx.L.mdz_get_velocity(ctx.h, mdz._dptr(uu), mdz._dptr(vv), mdz._dptr(pp)))
        x, z, ph, _, _ = ctx.get_markers()
        got = dict(u=uu, v=vv, p=pp - pp.mean(), sxxd=ctx.get_marker_attr(mdz.M_SXXD),
                   szzd=ctx.get_marker_attr(mdz.M_SZZD), sxz=ctx.get_marker_attr(mdz.M_SXZ), x=x, z=z)
        ctx.close()
        e = {k: (float(np.linalg.norm(got[k] - ref[k]) / max(np.linalg.norm(ref[k]), 1e-300))
                 if len(got[k]) == len(ref[k]) else None) for k in ref}
        e["phases_equal"] = bool(len(ph) == len(m["phase"]) and np.array_equal(ph, m["phase"]))
        e["nonlinear_its"] = r.nonlinear_its
        out[name] = e
    return out


def mlp_workload():
    """The local-rheology MLP on its own: 2^24 tuples of the lithosphere
    phases, one epoch of training at batch 65536, inference over 2^24 cells."""
    import mdz
    import mdz_setups
    cfg = mdz_setups.config_lithosphere(Nx=65, Nz=33)
    ctx = mdz_setups.load_context(cfg)
    n = 1 << 24
    ctx.mlp_init(1)
    t0 = time.perf_counter()
    ctx.mlp_generate(cfg["mat"], cfg["model"].rheo, n, 5, LO_MLP, HI_MLP)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = ctx.mlp_train(n // 65536, 65536, 2e-3)
    t_epoch = time.perf_counter() - t0
    ctx.mlp_set_engine(0)
    b = ctx.mlp_benchmark(65536, 5)               # tcgen05 inference and training (the default)
    ctx.mlp_set_engine(1)
    b1 = ctx.mlp_benchmark(65536, 5)              # warp-level mma.sync
    ctx.close()
    flops = 2.0 * (8 * 64 + 64 * 64 + 64 * 2)     # algorithmic FLOP per row of the forward pass (9472)
    return {"tuples": n, "batch": 65536, "generate_s": t_gen, "epoch_s": t_epoch, "loss": loss,
            "ms_infer_2^24": b["ms_infer"], "ms_train_step": b["ms_train_step"], "rms_error": b["rms_error"],
            "infer_tflops": flops * n / (b["ms_infer"] * 1e-3) / 1e12, "engine": "tcgen05",
            "mma_sync": {"ms_infer_2^24": b1["ms_infer"], "infer_tflops": flops * n / (b1["ms_infer"] * 1e-3) / 1e12,
                         "ms_train_step": b1["ms_train_step"], "rms_error": b1["rms_error"]}}


class GpuLocalPlacement:
    """Runs the enclosed code on the CPUs the kernel lists as local to the GPU
    (its PCI device's local_cpulist, intersected with the CPUs this process may
    use), so that the host arrays it first touches are placed on the GPU's
    NUMA node, as a caller of the library would place its marker arrays; the
    previous CPU set is restored on exit.  `info` records what was found."""

    def __init__(self, dev):
        self.dev, self.info, self.saved = dev, {}, None

    def __enter__(self):
        import torch
        allowed = os.sched_getaffinity(0)
        self.info = {"allowed_cpus": len(allowed)}
        p = torch.cuda.get_device_properties(self.dev)
        bus = getattr(p, "pci_bus_id", None)
        if bus is None:
            self.info["gpu_local_cpus"] = "unknown (no PCI id)"
            return self.info
        path = "/sys/bus/pci/devices/%04x:%02x:%02x.0" % (getattr(p, "pci_domain_id", 0) or 0, bus,
                                                           getattr(p, "pci_device_id", 0) or 0)
        try:
            text = open(path + "/local_cpulist").read().strip()
            node = open(path + "/numa_node").read().strip()
        except OSError:
            self.info["gpu_local_cpus"] = "unknown (%s unreadable)" % path
            return self.info
        local = set()
        for part in text.split(","):
            a, _, b = part.partition("-")
            if a:
                local.update(range(int(a), int(b or a) + 1))
        use = allowed & local
        self.info.update({"gpu_numa_node": node, "gpu_local_cpus": len(local), "used_cpus": len(use or allowed)})
        if use and use != allowed:
            self.saved = allowed
            os.sched_setaffinity(0, use)
        return self.info

    def __exit__(self, *exc):
        if self.saved is not None:
            os.sched_setaffinity(0, self.saved)
        return False


def e2e_form(cfg_builder, precision, learned, steps, size, warmup):
    """Same step through the public API with the marker state owned by the
    host, as in the reference's time loop: every step uploads the markers
    (positions, phases, the eight attributes), runs the step and downloads the
    advected markers, their velocities, the updated attributes and the grid
    velocity into the same host arrays, which the next step uploads again.
    The host arrays hold the run's marker capacity (reseeding changes the
    count from step to step) and are page-locked once with host_register (as
    a caller would register its marker arrays), so the copies are DMA
    transfers."""
    import numpy as np
    import mdz
    import mdz_setups
    cfg = cfg_builder(precision, learned, size)
    m = cfg["markers"]
    cap = marker_capacity(cfg)
    ctx = mdz_setups.load_context(cfg, max_markers=cap)
    model, mat = cfg["model"], cfg["mat"]
    if learned:
        train_guess(ctx, cfg)
    g = cfg["grid"]
    n = len(m["x"])
    attrs = ((mdz.M_SXXD, "sxxd"), (mdz.M_SZZD, "szzd"), (mdz.M_SXZ, "sxz"), (mdz.M_STRAIN_PL, "strain_pl"),
             (mdz.M_STRAIN, "strain"), (mdz.M_T, "T"), (mdz.M_CMUL, "cmul"), (mdz.M_P, "P"))
    hin = {"x": np.zeros(cap), "z": np.zeros(cap), "phase": np.full(cap, -1, np.int32)}   # the caller's arrays
    for _, key in attrs:
        hin[key] = np.zeros(cap)
    for key in hin:
        hin[key][:n] = m[key]
    hvx, hvz = np.zeros(cap), np.zeros(cap)
    hout = [hin["x"], hin["z"], hin["phase"], hvx, hvz]
    hu = np.empty(g.size(-1))
    pinned = list(hin.values()) + [hvx, hvz, hu]
    for a in pinned:
        mdz.host_register(a)
    times, parts, reps = [], [0.0, 0.0, 0.0, 0.0], []
    h2d = d2h = 0
    for step in range(warmup + steps):   # the same steps as the device-resident form; the last `steps` timed
        t0 = time.perf_counter()
        # one batched upload and one batched download per step (mdz_set/get_marker_state: the copies of a
        # call spread over several streams and copy engines)
        ctx.set_marker_state(hin["x"][:n], hin["z"][:n], hin["phase"][:n], {attr: hin[key][:n] for attr, key in attrs})
        t1 = time.perf_counter()
        rep = ctx.time_step(mat, model)
        t2 = time.perf_counter()
        n_in, n = n, ctx.n_markers
        reps.append({k: rep.as_dict()[k] for k in ("nonlinear_its", "linear_its", "ms_solve", "ms_rheology",
                                                    "ms_total", "markers_added")})
        ctx.get_marker_state(hout, {attr: hin[key] for attr, key in attrs})
        ctx.L.mdz_get_velocity(ctx.h, mdz._dptr(hu), None, None)
        t3 = time.perf_counter()
        if step < warmup:
            reps.pop()
            continue
        times.append((t3 - t0) * 1e3)
        h2d += (n_in * (8 * 2 + 4) + n_in * 8 * len(attrs)) / steps
        d2h += (n * (8 * 4 + 4) + n * 8 * len(attrs) + g.size(-1) * 8) / steps
        for q, v in enumerate(((t1 - t0) * 1e3, (t2 - t1) * 1e3, (t3 - t2) * 1e3, rep.ms_total)):
            parts[q] += v / steps
    for a in pinned:
        mdz.host_unregister(a)
    ctx.close()
    split = dict(zip(("upload_ms", "step_ms", "download_ms", "step_device_ms"), parts))
    split["reports"] = reps
    split["markers_final"] = n
    return sum(times) / len(times), int(h2d), int(d2h), split


def builder(size):
    import mdz_setups

    def b(precision, learned, sz=size):
        if sz:
            nx, nz = sz
            return mdz_setups.config_lithosphere(Nx=nx, Nz=nz, precision=precision, learned=learned)
        return mdz_setups.config_lithosphere(precision=precision, learned=learned)
    return b


# The CPU time step is sampled on the same model at 1/64 of the cells (same
# domain, layering, rheology, markers per cell and time step), scaled by the
# cell count to the full grid; SAMPLE_CHECK is a second resolution (1/16 of
# the cells) whose first steps test that scaling.
SAMPLE_GRID = (129, 65)
SAMPLE_CHECK = (257, 129)


def _cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


class CpuModel:
    """Consecutive oracle time steps (the restated reference functions in C,
    threaded over nodes and markers with OpenMP, plus SciPy SuperLU for each
    defect solve in place of CHOLMOD) of the lithosphere model at one grid
    size.  step() returns the wall time of one step in ms and its report."""

    def __init__(self, nx, nz):
        import mdz_setups
        self.cfg = mdz_setups.config_lithosphere(Nx=nx, Nz=nz, precision=64)
        c = self.cfg
        self.m = {k: v.copy() for k, v in c["markers"].items()}
        self.u, self.v, self.p = c["u"].copy(), c["v"].copy(), c["p"].copy()
        self.cells = (nx - 1) * (nz - 1)

    def step(self):
        import oracle_step
        c = self.cfg
        t0 = time.perf_counter()
        self.u, self.v, self.p, rep = oracle_step.time_step(c["grid"], c["mat"], c["model"], self.m, self.u, self.v,
                                                            self.p)
        return (time.perf_counter() - t0) * 1e3, rep


def cpu_sample(steps, warmup, size=None, check=True):
    """CPU reference time per full-grid step: `warmup` untimed and `steps`
    timed consecutive steps of the model at SAMPLE_GRID (the same step indices
    as the GPU forms time), scaled by cells; then the first two steps at
    SAMPLE_CHECK against the first two at SAMPLE_GRID, per cell."""
    nx, nz = size if size else (1025, 513)
    full = (nx - 1) * (nz - 1)
    os.environ.setdefault("OMP_NUM_THREADS", str(_cpu_threads()))
    a = CpuModel(*SAMPLE_GRID)
    scale = full / a.cells
    first, times, reps = [], [], []
    for k in range(warmup + steps):
        ms, rep = a.step()
        if k < 2:
            first.append(ms)
        if k >= warmup:
            times.append(ms)
            reps.append(rep["nonlinear_its"])
    value = scale * sum(times) / len(times)
    out = dict(value=value, unit=UNIT, cores=int(os.environ["OMP_NUM_THREADS"]), kind="port",
                sample=("%d consecutive time steps (after %d untimed) of the same lithosphere model at %dx%d "
                        "(%d cells, 16 markers per cell), scaled by cells x%.0f to %dx%d; oracle C functions "
                        "threaded with OpenMP, defect solves by SciPy SuperLU on one thread (CHOLMOD unavailable)"
                        % (steps, warmup, SAMPLE_GRID[0], SAMPLE_GRID[1], a.cells, scale, nx, nz)),
                sample_step_ms=times, sample_nonlinear_its=reps)
    if check:
        b = CpuModel(*SAMPLE_CHECK)
        t2 = [b.step()[0] for _ in range(2)]
        per_cell_a = sum(first) / a.cells
        per_cell_b = sum(t2) / b.cells
        out["scaling_check"] = {"grid": "%dx%d" % SAMPLE_CHECK, "first_two_steps_ms": t2, "ms_per_cell": per_cell_b,
                                "ms_per_cell_at_%dx%d" % SAMPLE_GRID: per_cell_a, "ratio": per_cell_b / per_cell_a}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", default=None, help="NXxNZ override (tests only)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mlp", action="store_true")
    ap.add_argument("--forms", default="both", choices=["both", "fast"],
                    help="fast: run only the learned FP32-refined form and print nothing (profiling)")
    ap.add_argument("--guess-steps", type=int, default=3000, help="Adam steps of the learned guess")
    ap.add_argument("--mlp-only", action="store_true",
                    help="run only the MLP workload (2^24 tuples, one epoch, inference) and print its object")
    args = ap.parse_args()
    rank, world, local = _dist()
    size = tuple(int(s) for s in args.size.split("x")) if args.size else None
    if args.impl == "reference":
        if rank != 0:
            return 0
        ref = cpu_sample(args.steps, args.warmup, size)
        val = ref["value"]
        line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": val, "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "lithosphere %s, 4 phases, 16 markers/cell, one Newton time step"
                                       % ("x".join(map(str, size)) if size else "1025x513"),
                           "timed": "each step is one time step of the model at %dx%d, scaled by cells"
                                    % SAMPLE_GRID},
                "cpu_baseline": ref,
                "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import mdz
    mdz.load_library()
    if args.mlp_only:
        print(json.dumps(mlp_workload()))
        return 0
    b = builder(size)
    if world > 1:
        torch.distributed.barrier()
    hbm, bf16, peak_kind = peaks()
    if args.forms == "fast":   # profiling runs: the learned FP32-refined form alone, short guess training
        GUESS_STEPS[0] = args.guess_steps
        run_form(b, 32, 1, args.steps, args.warmup, size)
        return 0
    GUESS_STEPS[0] = args.guess_steps
    with ClockSampler(local) as clk:
        plain = run_form(b, 64, 0, args.steps, args.warmup, size)
        fast = run_form(b, 32, 1, args.steps, args.warmup, size, reseed=rank == 0 and not args.no_cpu)
    ms = fast["ms_wall"]
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    with GpuLocalPlacement(torch.cuda.current_device()) as placement:
        e2e_ms, h2d, d2h, e2e_split = e2e_form(b, 32, 1, args.steps, size, args.warmup)
    e2e_split["host_placement"] = placement
    k = fast["kernel"]
    achieved = k["bytes"] / (k["ms"] * 1e-3) / 1e9 if k["ms"] > 0 else None
    line = {
        "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic",
        "config": {"workload": "lithosphere %s, 4 phases, 16 markers/cell, one Newton time step"
                               % ("x".join(map(str, size)) if size else "1025x513"),
                   "markers": len(fast["cfg"]["markers"]["x"]),
                   "l2": "inputs larger than L2 (markers %.0f MB)" % (len(fast["cfg"]["markers"]["x"]) * 84 / 1e6),
                   "parallelism": "replicas" if world > 1 else "single"},
        "forms": {"plain_fp64_ms": plain["ms_wall"], "learned_fp32_ir_ms": fast["ms_wall"],
                  # wall time of each timed step and its device time (CUDA events inside the step)
                  "plain_step_ms": plain["step_ms"], "learned_fp32_ir_step_ms": fast["step_ms"],
                  "plain_step_device_ms": [r["ms_total"] for r in plain["reports"]],
                  "learned_fp32_ir_step_device_ms": [r["ms_total"] for r in fast["reports"]],
                  "speedup_vs_plain_fp64": plain["ms_wall"] / fast["ms_wall"],
                  "plain_report": plain["reports"][-1], "learned_fp32_ir_report": fast["reports"][-1],
                  "guess_training_s": fast["train"][0], "guess_training_loss": fast["train"][1],
                  "plain_fp64_classes": plain["kernel"]["classes"], "learned_fp32_ir_classes": fast["kernel"]["classes"],
                  # relative 2-norm difference of each output field after the same steps (pressure
                  # with its mean removed: the operator leaves it undetermined)
                  "field_rel_diff_fp32_vs_fp64": field_diffs(fast["final"], plain["final"])},
        "e2e": {"value": e2e_ms, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "split": e2e_split},
        "gpu_launches": fast["launches"] // args.steps,
        "roofline": {"bound": "hbm", "kernel": k["name"], "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None,
                     "traffic": TRAFFIC_PER_LAUNCH.get(k["name"]) if not size else None,
                     "peak_kind": peak_kind},
        # every instrumented kernel class of the FP32 form: live CUDA-event time per step, algorithmic
        # bytes over that time and its fraction of the measured copy bandwidth
        "class_bandwidth": {name: {"ms_per_step": c["ms"] / args.steps, "GB/s": c["bytes"] / (c["ms"] * 1e-3) / 1e9,
                                   "frac": c["bytes"] / (c["ms"] * 1e-3) / 1e9 / hbm}
                            for name, c in fast["kernel"]["classes"].items() if c["ms"] > 0},
        "clocks": clk.summary(),
    }
    if fast["reseed"]:
        line["reseed"] = fast["reseed"]
    if rank == 0 and not args.no_mlp:
        line["mlp"] = mlp_workload()
    if rank == 0 and not args.no_cpu:
        line["field_rel_err_vs_oracle"] = parity_vs_oracle()
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(3, 0, size, check=False)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Benchmark of the GB300 glasma leapfrog (one JSON line on rank 0).

Workload: the production-size plain method, a 128x128x512 lattice (open z, a=1,
dt=0.125a) advanced by the real-time SU(3) leapfrog Dynamics::SUNc::Update.  One
"step" is one full leapfrog step of the whole lattice; the metric is
site-updates/s (lattice sites x steps / second).

  value     FP64, fields resident in HBM, CUDA events around K steps
  e2e       FP64 through the C ABI with host buffers: every step uploads the six
            dynamical fields from pinned host memory in the reference's host layout,
            steps, and reads the bulk energy back
  fp32      the same lattice in FP32 storage/arithmetic with FP64 reductions and
            reunitarisation every 16 steps, with its energy error against FP64
  roofline  for the dominant kernel (the electric-field kernel K1), per-launch CUDA events
  cpu_baseline  the oracle's CPU restatement on the host cores on a bounded slab

`--impl reference` times the reference algorithm on the host CPU (the oracle port,
all host threads) on a slab of the same workload and prints the same metric.

Inputs are seeded synthetic fields with the workload's shapes: links
exp(i 0.3 t^a r^a), E ~ N(0, 0.1^2), currents ~ N(0, 0.02^2), r ~ N(0,1).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_WORK = (128, 128, 512)
A_WORK = (1.0, 1.0, 1.0)
DT = 0.125
SEED = 1002
LINK_AMP, E_AMP, J_AMP = 0.3, 0.1, 0.02
INPUT_FIELDS = ("U", "E", "Jp", "Jm", "JpStat", "JmStat")
# compulsory HBM bytes per site of each kernel (read + write of what it must touch once)
# ("fp32_l12": FP32 with 12-real links, rows 0 and 1 of each link read and written, 144 B per site)
KERNEL_BYTES = {
    "efield_jstat": {"fp64": 432 + 2 * 192 + 128 + 2 * 128, "fp32": 216 + 2 * 96 + 64 + 2 * 64,
                     "fp32_l12": 144 + 2 * 96 + 64 + 2 * 64},
    "links_j": {"fp64": 192 + 2 * 432 + 128 + 2 * 128, "fp32": 96 + 2 * 216 + 64 + 2 * 64,
                "fp32_l12": 96 + 2 * 144 + 64 + 2 * 64},
    "fused_step": {"fp64": 1760, "fp32": 880, "fp32_l12": 736},  # one pass: every per-site array read and written once
    "march_step": {"fp64": 1760, "fp32": 880, "fp32_l12": 736},  # the marching plaquette step, likewise
    # plaquette method: the same compulsory state traffic as K1 / K2 (the 48 contribution reals per site
    # the force kernel hands to the link kernel are an intermediate of this method, not algorithmic
    # bytes; ncu's DRAM traffic shows what they cost)
    "plaquette_forces": {"fp64": 1200, "fp32": 600, "fp32_l12": 528},
    "links_gather": {"fp64": 1440, "fp32": 720, "fp32_l12": 576},
}
STEP_BYTES = {"fp64": 1760, "fp32": 880, "fp32_l12": 736}  # every per-site state array read and written once
FALLBACK_HBM_GBS = 6800.0


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        for k in ("hbm_gbs", "hbm_GBs", "hbm"):
            if k in d:
                v = d[k]
                if isinstance(v, dict):
                    v = v.get("value", v.get("burst"))
                return float(v), "measured"
    except Exception:
        pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic():
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        return json.load(open(p))
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in getattr(self, "lines", []):
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- inputs
def device_inputs(torch, N, seed, dev):
    """Seeded synthetic fields in the reference's host layout (FP64), generated on the device."""
    Nx, Ny, Nz = N
    S = Nx * Ny * (Nz + 2)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    inv3 = 1.0 / 3.0 ** 0.5
    U = torch.empty((S, 3, 3, 3), dtype=torch.complex128, device=dev)
    Uf = U.view(S * 3, 3, 3)
    chunk = 1 << 22
    for c0 in range(0, S * 3, chunk):
        c1 = min(S * 3, c0 + chunk)
        al = LINK_AMP * torch.randn((c1 - c0, 8), generator=g, device=dev, dtype=torch.float64)
        H = torch.zeros((c1 - c0, 3, 3), dtype=torch.complex128, device=dev)
        H[:, 0, 0] = 0.5 * (al[:, 2] + al[:, 7] * inv3)
        H[:, 1, 1] = -0.5 * (al[:, 2] - al[:, 7] * inv3)
        H[:, 2, 2] = -al[:, 7] * inv3
        H[:, 1, 0] = 0.5 * torch.complex(al[:, 0], al[:, 1])
        H[:, 2, 0] = 0.5 * torch.complex(al[:, 3], al[:, 4])
        H[:, 2, 1] = 0.5 * torch.complex(al[:, 5], al[:, 6])
        H[:, 0, 1] = H[:, 1, 0].conj()
        H[:, 0, 2] = H[:, 2, 0].conj()
        H[:, 1, 2] = H[:, 2, 1].conj()
        M = torch.linalg.matrix_exp(1j * H)  # [i, j]
        Uf[c0:c1] = M.transpose(-1, -2)      # host layout stores element (i,j) at i + 3j
        del al, H, M
    f = {"U": U.view(Nz + 2, Ny, Nx, 3, 3, 3)}
    f["E"] = E_AMP * torch.randn((Nz + 2, Ny, Nx, 3, 8), generator=g, device=dev, dtype=torch.float64)
    for k in ("Jp", "Jm", "JpStat", "JmStat"):
        f[k] = J_AMP * torch.randn((Nz + 2, Ny, Nx, 8), generator=g, device=dev, dtype=torch.float64)
    for v in f.values():  # open-z ghost slices in sync
        v[0] = v[1]
        v[-1] = v[-2]
    return f


def host_slab(fields_dev, nz_slab):
    """First nz_slab z-slices (plus ghosts) of the device inputs, as numpy arrays."""
    out = {}
    for k, v in fields_dev.items():
        a = v[: nz_slab + 2].cpu().numpy().copy()
        a[-1] = a[-2]
        out[k] = a
    import numpy as np

    out["UOld"] = out["U"].copy()
    return {k: np.ascontiguousarray(v) for k, v in out.items()}


def numpy_inputs(N, seed):
    """Same distribution as device_inputs, generated on the host (reference arm)."""
    import numpy as np

    from oracle import oracle as O

    f = O.random_fields(N, seed, link_amp=LINK_AMP, e_amp=E_AMP, j_amp=J_AMP)
    return {k: np.ascontiguousarray(v) for k, v in f.items()}


# ----------------------------------------------------------------------------- CPU legs
# Both CPU legs time the same bounded sample of the workload: full leapfrog steps (SaveOldLink included,
# as Dynamics::SUNc::Update does) of a 128x128x32 slab of the lattice, on all host threads.
CPU_SLAB_NZ = 32


def cpu_impl():
    """'reference' where the reference's own code compiled here (oracle/_ref, built only where the
    reference checkout exists), else 'port' (the oracle restatement, built everywhere)."""
    from oracle import build as ob

    return "reference" if ob.reference_source_dir() and ob.build_reference() else "port"


class CpuStepper:
    """One full leapfrog step of a slab on the host CPU, by the reference's own compiled code or by the
    oracle restatement; `threads` = the OpenMP threads it runs on."""

    def __init__(self, fields, N, impl):
        from oracle import oracle as O

        self.impl, self.N = impl, N
        threads = os.cpu_count() or 1
        if impl == "reference":
            self.ref = O.Reference(N, A_WORK, threads=threads)
            self.ref.set_fields(fields)
            self.threads = threads
        else:
            self.orc = O.Oracle(threads=threads)
            self.fields = fields
            self.threads = self.orc.threads()

    def step(self):
        if self.impl == "reference":
            self.ref.update(1, DT)
        else:
            self.orc.update(self.fields, self.N, A_WORK, DT, 1, save_uold=True)


def cpu_sample_desc(n, secs, threads, impl):
    who = "the reference's own code compiled from its sources" if impl == "reference" else "oracle restatement"
    return ("%s leapfrog steps (Dynamics::SUNc::Update incl. SaveOldLink) of a %dx%dx%d slab of the workload%s, "
            "%s, %d threads" % (n, N_WORK[0], N_WORK[1], CPU_SLAB_NZ, "" if secs is None else " in %.1f s" % secs,
                               who, threads))


def time_cpu(fields, min_seconds, max_steps, impl):
    slab = (N_WORK[0], N_WORK[1], CPU_SLAB_NZ)
    st = CpuStepper(fields, slab, impl)
    st.step()  # warm-up
    t0 = time.perf_counter()
    n = 0
    while n < max_steps:
        st.step()
        n += 1
        if time.perf_counter() - t0 > min_seconds:
            break
    dt = time.perf_counter() - t0
    return slab[0] * slab[1] * slab[2] * n / dt, n, dt, st.threads


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    slab = (N_WORK[0], N_WORK[1], CPU_SLAB_NZ)
    impl = cpu_impl() if args.cpu_impl == "auto" else args.cpu_impl
    st = CpuStepper(numpy_inputs(slab, SEED), slab, impl)
    for _ in range(args.warmup):
        st.step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        st.step()
        times.append(time.perf_counter() - t0)
    sites = slab[0] * slab[1] * slab[2]
    ms = 1e3 * sum(times) / len(times)
    value = sites / (ms * 1e-3)
    line = {
        "impl": "reference",
        "metric": "leapfrog site-updates/s",
        "value": value,
        "unit": "site-updates/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": DATA_DESC,
        "config": workload_config(world),
        "sample": {"lattice": list(slab), "note": "each step is one full leapfrog step of this slab of the "
                                                  "workload's lattice; site-updates/s are per slab site"},
        "cpu_baseline": {"value": value, "unit": "site-updates/s", "cores": st.threads, "kind": impl,
                         "sample": cpu_sample_desc("each of %d" % args.steps, None, st.threads, impl)},
        "e2e": {"value": value, "unit": "site-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(world):
    """The config object both arms print (identical, so the two lines describe one workload)."""
    N = N_WORK
    return {"workload": "glasma leapfrog %dx%dx%d FP64 (plain method, production size)" % N,
            "lattice": list(N), "dt": DT, "a": list(A_WORK), "parallelism": "replicas" if world > 1 else "1 GPU",
            "l2": "inputs larger than L2 (%.1f GB of FP64 state)" % (STEP_BYTES["fp64"] / 2 * N[0] * N[1] * N[2] / 1e9)}


DATA_DESC = "synthetic (seeded SU(3) links exp(i 0.3 t.r), E ~ N(0,0.01), J ~ N(0,4e-4); workload shapes)"


# ----------------------------------------------------------------------------- GPU leg
def run_ours(args):
    import numpy as np
    import torch

    rank, world, local = env_rank()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from soerenpragya3dglasma_gb300 import Lattice, build

    if rank == 0:
        build.build()
    if world > 1:
        dist.barrier()

    def barrier():
        if world > 1:
            dist.barrier()

    # a stream of our own: the legacy default stream is handle 0, which the C ABI reads as
    # "the handle's own stream", and the CUDA events below must sit on the launching stream
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    N = N_WORK
    vol = N[0] * N[1] * N[2]
    inputs = device_inputs(torch, N, SEED + rank, dev)
    torch.cuda.synchronize()

    tiles = {}

    def make_lattice(precision, link_reals=18):
        lat = Lattice(N, A_WORK, precision=precision, reunitarize_every=16 if precision == "fp32" else 0,
                      stream=stream)
        lat.set_step_method(args.step_method if precision == "fp64" else (args.fp32_step_method or args.step_method))
        if args.march_chunk:
            lat.set_march_chunk(args.march_chunk)
        lat.link_reals = link_reals
        if precision == "fp64":
            lat.fp64_arithmetic = args.fp64_arith
        for k in INPUT_FIELDS:
            lat.upload_device(k, inputs[k].data_ptr())
        lat.upload_device("UOld", inputs["U"].data_ptr())
        if args.tile:
            lat.set_tile(args.tile)
            tiles[precision + ("_l12" if link_reals == 12 else "")] = args.tile
        else:  # untimed: picks the electric-field kernel's block tile
            tiles[precision + ("_l12" if link_reals == 12 else "")] = lat.autotune(DT)
        return lat

    peak, peak_kind = hbm_peak()
    traffic = ncu_traffic()

    def roofline(name, prec, ms):
        alg = KERNEL_BYTES[name][prec] * vol
        ach = alg / (ms * 1e-3) / 1e9
        key = "%s_%s" % (name, prec)
        tr = traffic.get(key)
        # what limits the kernel, from the ncu capture of the same kernel: the FP64 kernels keep GB300's
        # FP64 pipe >90 % busy (hence their small HBM fraction), the FP32 ones are bound by HBM traffic
        # and issue
        pa = traffic.get("pipe_active", {}).get(key)
        bound = "fp64_pipe" if pa and pa.get("pipe") == "fp64" and pa.get("frac", 0) > 0.8 else "hbm"
        out = {"bound": bound, "kernel": name, "achieved": ach, "peak": peak, "unit": "GB/s",
               "frac": ach / peak, "peak_kind": peak_kind, "traffic": tr,
               "algorithmic_bytes_per_launch": alg, "launch_ms": ms,
               "pipe_active": pa.get("frac") if pa else None, "pipe": pa.get("pipe") if pa else None,
               "pipe_source": traffic.get("sources", {}).get(key)}
        return out

    def max_over_ranks(x):
        if world > 1:
            t = torch.tensor([x], device=dev, dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return x

    def time_observables(lat, reps=3):
        """CUDA-event milliseconds of one bulk-energy and one Gauss-law measurement (each returns to
        the host, as the reference's measurement steps do)."""
        out = {}
        for name, fn in (("bulk", lat.bulk), ("gauss", lat.gauss)):
            fn()
            torch.cuda.synchronize()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(reps):
                fn()
            t1.record(stream)
            torch.cuda.synchronize()
            out[name] = t0.elapsed_time(t1) / reps
        return out

    # FP32 links are reunitarised every 16 steps: its timed window is a multiple of 16 steps, so it
    # holds its share of reunitarisations whatever the alignment.
    steps32 = 16 * max(1, -(-args.steps // 16))

    def timed_run(precision, sampler=None, nsteps=None, link_reals=18):
        nsteps = nsteps or args.steps
        lat = make_lattice(precision, link_reals)
        lat.step(DT, args.warmup, save_uold=False)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if sampler is not None:
            sampler.__enter__()
        e0.record(stream)
        kms = lat.step_profiled(DT, nsteps, save_uold=False)
        e1.record(stream)
        torch.cuda.synchronize()
        if sampler is not None:
            sampler.__exit__(None, None, None)
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1)) / nsteps
        if lat.last_step_method == "one_pass":
            kern = {"fused_step": kms[0] / nsteps}
        elif lat.last_step_method == "march":
            kern = {"march_step": kms[0] / nsteps}
        elif lat.last_step_method == "plaquette":
            kern = {"plaquette_forces": kms[0] / nsteps, "links_gather": kms[1] / nsteps}
        else:
            kern = {"efield_jstat": kms[0] / nsteps, "links_j": kms[1] / nsteps}
        return lat, ms, kern

    run64 = args.only in ("both", "fp64")
    run32 = args.only in ("both", "fp32")
    clk = ClockSampler(local)
    lat = None
    value = ms_step = rl = k_ms = e64 = obs64 = None
    if run64:
        # ---- FP64, resident fields (the headline)
        lat, ms_step, k_ms = timed_run("fp64", clk)
        value = world * vol / (ms_step * 1e-3)
        if run32 and steps32 > args.steps:  # untimed: bring the FP64 state to the FP32 leg's step count
            lat.step(DT, steps32 - args.steps, save_uold=False)
        e64 = lat.bulk()
        obs64 = time_observables(lat)
        dom = max(k_ms, key=k_ms.get)
        rl = roofline(dom, "fp64", k_ms[dom])

    gauge = None
    if run64 and not args.no_gauge:
        # ---- Coulomb gauge fixing (the production workload's last stage) on an evolved MV collision:
        # iterations/s, iterations until theta = avg deviation^2 < 1e-10, and FFT GB/s
        import numpy as np

        from soerenpragya3dglasma_gb300 import GlasmaError

        alpha_ref = 0.96  # alpha = 0.08 in the p^2_max/p^2 normalisation, times p^2_max = 12 at a = 1
        zrng = np.random.default_rng(SEED - 1)
        zl, zr = zrng.standard_normal(8 * N[0] * N[1]), zrng.standard_normal(8 * N[0] * N[1])
        centres = (N[2] // 2 - 3 * N[2] // 16, N[2] // 2 + 3 * N[2] // 16)  # 256 -+ 96 at Nz = 512
        glat = Lattice(N, A_WORK, stream=stream)
        glat.mv_init(zl, zr, qs=(0.5, 0.5), centers=centres, sigma=N[2] / 64.0, lam=1.65, meff=0.2, dt=DT)
        glat.step(DT, args.gauge_evolve, save_uold=False)
        torch.cuda.synchronize()

        def time_gauge(fft_fp32, open_z, mixed=False, iters=None):
            glat.gauge_reset()
            torch.cuda.synchronize()
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            try:
                log = glat.coulomb_fix(alpha_ref, iters or args.gauge_iters, tol=1e-15, fft_fp32=fft_fp32,
                                       open_z=open_z, mixed=mixed)
                err = None
            except GlasmaError as e:
                log, err = e.log, str(e)
            g1.record(stream)
            torch.cuda.synchronize()
            out = {"open_z": open_z}
            if err is not None:  # the reference's own iteration exits on its unitarity guard here
                out.update({"exited_on_guard": True, "iterations_before_exit": len(log), "error": err})
                if not len(log):
                    return out
            theta = log[:, 2] ** 2
            hit = np.nonzero(theta < 1e-10)[0]
            out.update({"iterations_per_s": len(log) / (g0.elapsed_time(g1) * 1e-3),
                        "ms_per_iteration": g0.elapsed_time(g1) / len(log), "iterations_run": len(log),
                        "seconds": g0.elapsed_time(g1) * 1e-3,
                        "iterations_to_theta_1e-10": int(hit[0]) + 1 if len(hit) else None,
                        "theta_first": float(theta[0]), "theta_last": float(theta[-1]),
                        "max_deviation_last": float(log[-1, 1])})
            if mixed:  # the FP32 sweeps hand over at the first row with max |Delta| <= 1e-5 (or on a stall)
                below = np.nonzero(log[:, 1] <= 1e-5)[0]
                out["fp32_sweeps_to_max_deviation_1e-5"] = int(below[0]) + 1 if len(below) else None
            return out

        def time_fft(fp32):
            X = torch.randn((8, N[2], N[1], N[0]), dtype=torch.complex64 if fp32 else torch.complex128, device=dev)
            Y = torch.empty_like(X)
            glat.fft3d_device(X.data_ptr(), Y.data_ptr(), fp32=fp32)
            torch.cuda.synchronize()
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            for _ in range(5):
                glat.fft3d_device(X.data_ptr(), Y.data_ptr(), fp32=fp32)
            f1.record(stream)
            torch.cuda.synchronize()
            ms = f0.elapsed_time(f1) / 5
            # three axis passes, each reads and writes the 8-colour array once
            return ms, 3 * 2 * (8 if fp32 else 16) * 8 * vol / (ms * 1e-3) / 1e9

        def time_local(alg, param):
            # the reference's two local updates (Los Alamos: checkerboard passes with the Cabibbo-Marinari
            # max-trace projection; Jacobi: every site at once) on the same state
            glat.gauge_reset()
            torch.cuda.synchronize()
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            log = glat.coulomb_fix(param, args.local_gauge_iters, tol=0.0, algorithm=alg)
            g1.record(stream)
            torch.cuda.synchronize()
            return {"param": param, "ms_per_iteration": g0.elapsed_time(g1) / len(log), "iterations_run": len(log),
                    "max_deviation_first": float(log[0, 1]), "max_deviation_last": float(log[-1, 1]),
                    "functional_last": float(log[-1, 6])}

        # the reference's iteration leaves SU(3) on this open-z state and exits on its guard; the open-z
        # functional (GLASMA_GF_OPEN_Z) converges: theta < 1e-10 is timed with it
        runs = {"reference_semantics": time_gauge(False, False)}
        for fft_fp32 in (False, True):
            r = time_gauge(fft_fp32, True)
            if r.get("iterations_to_theta_1e-10"):  # every iteration costs the same
                r["seconds_to_theta_1e-10"] = r["iterations_to_theta_1e-10"] * r["ms_per_iteration"] * 1e-3
            runs["fft_fp32" if fft_fp32 else "fft_fp64"] = r
        # FP32 sweeps first, FP64 for the final ones (GLASMA_GF_MIXED); the two phases cost differently,
        # so the time to theta < 1e-10 is taken by a second run stopped there
        r = time_gauge(False, True, mixed=True)
        r["mixed"] = "FP32 sweeps until max |Delta| <= 1e-5 (or stalled), then FP64 sweeps"
        if r.get("iterations_to_theta_1e-10"):
            r["seconds_to_theta_1e-10"] = time_gauge(False, True, mixed=True,
                                                     iters=r["iterations_to_theta_1e-10"])["seconds"]
        runs["mixed_fp32_fp64"] = r
        if args.local_gauge_iters > 0:
            runs["los_alamos"] = time_local("los_alamos", 0.0)
            runs["jacobi"] = time_local("jacobi", 0.3)
        fft_ms, fft_gbs = time_fft(False)
        fft32_ms, fft32_gbs = time_fft(True)
        gauge = {"state": "MV collision (seeded charges, g^2 mu 0.5, m 0.2, sigma_z %g, centres %d/%d) evolved %d "
                          "steps" % (N[2] / 64.0, centres[0], centres[1], args.gauge_evolve),
                 "alpha_reference": alpha_ref, **runs,
                 "fft3d_ms": fft_ms, "fft_gbs": fft_gbs, "fft3d_fp32_ms": fft32_ms, "fft_fp32_gbs": fft32_gbs,
                 "fft_note": "one 3D FFT of 8 colour planes, device to device, including one copy into and one "
                             "out of the work array; the gauge iteration transforms 4 packed colour-pair planes "
                             "twice"}
        del glat

    fp32 = None
    if run32:
        # ---- FP32 on the same inputs
        lat32, ms32, k32 = timed_run("fp32", None if run64 else clk, steps32)
        e32 = lat32.bulk()
        obs32 = time_observables(lat32)
        dom32 = max(k32, key=k32.get)
        fp32 = {"value": world * vol / (ms32 * 1e-3), "ms_per_step": ms32,
                "step_hbm_frac": STEP_BYTES["fp32"] * vol / (ms32 * 1e-3) / 1e9 / peak,
                "energy_rel_err_vs_fp64": (abs(e32[9] - e64[9]) / abs(e64[9])) if e64 is not None else None,
                "steps": steps32, "reunitarisations_timed": steps32 // 16,
                "steps_compared": args.warmup + steps32,
                "kernel_ms": k32,
                "observables_ms": obs32,
                "roofline": roofline(dom32, "fp32", k32[dom32])}
        del lat32
        # ---- FP32 with 12-real links (rows 0 and 1 stored, row 2 = conj(row0 x row1)), same inputs
        lat12, ms12, k12 = timed_run("fp32", None, steps32, link_reals=12)
        e12 = lat12.bulk()
        dom12 = max(k12, key=k12.get)
        fp32["links12"] = {
            "value": world * vol / (ms12 * 1e-3), "ms_per_step": ms12,
            "step_bytes_per_site": STEP_BYTES["fp32_l12"],
            "step_hbm_frac": STEP_BYTES["fp32_l12"] * vol / (ms12 * 1e-3) / 1e9 / peak,
            "energy_rel_err_vs_fp64": (abs(e12[9] - e64[9]) / abs(e64[9])) if e64 is not None else None,
            "kernel_ms": k12, "roofline": roofline(dom12, "fp32_l12", k12[dom12]),
            "note": "one row-2 completion pass per step() call is inside ms_per_step"}
        del lat12

    if fp32 is not None and run64 and not args.no_gauge:
        # ---- FP32 against FP64 on a physical state: a 64x64x256 MV collision (seeded charges), 200 steps
        # from the same FP32-rounded initial fields.  The synthetic inputs above have strong fields;
        # this state has weak-field regions, where FP32 links near the identity are the hard case.
        import numpy as np

        Np, stepsp = (64, 64, 256), 200
        zrng = np.random.default_rng(1004)
        zl, zr = zrng.standard_normal(8 * Np[0] * Np[1]), zrng.standard_normal(8 * Np[0] * Np[1])
        with Lattice(Np, stream=stream) as lp:
            lp.mv_init(zl, zr, qs=(0.5, 0.5), centers=(128 - 24, 128 + 24), sigma=4.0, lam=1.65, meff=0.2, dt=DT)
            fp = lp.download_fields()
        fr = {k: (v.astype(np.complex64).astype(np.complex128) if np.iscomplexobj(v)
                  else v.astype(np.float32).astype(np.float64)) for k, v in fp.items()}
        vals = {}
        # fp64_exact: FP64 from the unrounded state, the chaos control -- how far two FP64 runs whose
        # starts differ only by FP32 rounding drift apart, the floor any FP32 run is measured against
        for prec, reals in (("fp64", 18), ("fp64_exact", 18), ("fp32", 18), ("fp32_l12", 12)):
            with Lattice(Np, precision=prec[:4], reunitarize_every=16 if prec.startswith("fp32") else 0,
                         stream=stream) as lp:
                lp.link_reals = reals
                lp.upload_fields(fp if prec == "fp64_exact" else fr)
                lp.step(DT, stepsp, save_uold=False)
                vals[prec] = (lp.bulk()[9], lp.objective(112, 144, Lattice.PL_OVER_PT), lp.unitarity()[0])
        fp32["physical_check"] = {
            "state": "MV collision 64x64x256 (g^2 mu 0.5, m 0.2, sigma_z 4, centres 104/152), %d steps, FP32 "
                     "reunitarised every 16 steps, both from the same FP32-rounded fields" % stepsp,
            "energy_rel_err_vs_fp64": abs(vals["fp32"][0] - vals["fp64"][0]) / abs(vals["fp64"][0]),
            "chaos_floor_energy_rel": abs(vals["fp64_exact"][0] - vals["fp64"][0]) / abs(vals["fp64"][0]),
            "chaos_floor_note": "FP64 from the unrounded state against FP64 from the FP32-rounded state",
            "pl_over_pt_central_fp64": vals["fp64"][1], "pl_over_pt_central_fp32": vals["fp32"][1],
            "fp32_unitarity_max": vals["fp32"][2],
            "links12_energy_rel_err_vs_fp64": abs(vals["fp32_l12"][0] - vals["fp64"][0]) / abs(vals["fp64"][0]),
            "links12_pl_over_pt_central": vals["fp32_l12"][1], "links12_unitarity_max": vals["fp32_l12"][2]}

    e2e = None
    if lat is not None and not args.no_e2e:
        # ---- e2e through the C ABI with pinned host buffers
        host = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in inputs.items()}
        for k in host:
            host[k].copy_(inputs[k])
        e2e_steps = max(1, min(args.steps, 10))
        h2d = sum(host[k].numel() * host[k].element_size() for k in INPUT_FIELDS)
        lat.upload("U", host["U"])
        torch.cuda.synchronize()
        barrier()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        # every step's inputs cross from pinned host memory inside the timed region; with
        # glasma_upload_begin/_finish the next step's inputs travel (copy engines, transfer stream)
        # while the current step's kernels run, and are converted into the fields after it
        for k in INPUT_FIELDS:
            lat.upload_begin(k, host[k])
        lat.upload_finish()
        for i in range(e2e_steps):
            if i + 1 < e2e_steps:
                for k in INPUT_FIELDS:
                    lat.upload_begin(k, host[k])
            lat.step(DT, 1, save_uold=False)
            lat.bulk()  # device -> host read of the step's energy (7 doubles); synchronises
            lat.upload_finish()
        a1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = max_over_ranks(a0.elapsed_time(a1)) / e2e_steps
        e2e = {"value": world * vol / (e2e_ms * 1e-3), "unit": "site-updates/s", "ms_per_step": e2e_ms,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 7 * 8, "steps": e2e_steps,
               "per_step": "upload U,E,Jp,Jm,JpStat,JmStat from pinned host (reference layout) + 1 step + bulk read; "
                           "the next step's uploads overlap the current step (glasma_upload_begin/_finish)"}

    # ---- CPU baseline (rank 0 at N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        hs = host_slab(inputs, CPU_SLAB_NZ)
        impl = cpu_impl() if args.cpu_impl == "auto" else args.cpu_impl
        rate, n, secs, threads = time_cpu(hs, 10.0, 50, impl)
        cpu = {"value": rate, "unit": "site-updates/s", "cores": threads, "kind": impl,
               "sample": cpu_sample_desc(n, secs, threads, impl)}
    del lat
    if world > 1:
        dist.destroy_process_group()
    if rank != 0:
        return
    line = {
        "metric": "leapfrog site-updates/s",
        "value": value,
        "unit": "site-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": DATA_DESC,
        "config": workload_config(world),
        "step_hbm_frac": (STEP_BYTES["fp64"] * vol / (ms_step * 1e-3) / 1e9 / peak) if ms_step else None,
        "gauge_fixing": gauge,
        "fp32": fp32,
        "roofline": rl,
        "kernel_ms": k_ms,
        "observables_ms": obs64,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        # per step: the one-pass kernel (or K1 + K2); per step() call: one ghost-slice sync
        "gpu_launches": (1 if ("fused_step" in (k_ms or {}) or "march_step" in (k_ms or {})) else 2) * args.steps + 1,
        "step_method": args.step_method,
        "fp32_step_method": args.fp32_step_method or args.step_method,
        "fp64_arithmetic": args.fp64_arith,
        "tiles": tiles,
    }
    if fp32 is not None:  # the FP32 figures once more, compactly, at the end of the line
        phys = fp32.get("physical_check") or {}
        line["fp32_headline"] = {
            "fp32_value": fp32["value"], "fp32_ms_per_step": fp32["ms_per_step"],
            "fp32_hbm_frac": fp32["step_hbm_frac"], "fp32_energy_rel_err": fp32["energy_rel_err_vs_fp64"],
            "fp32_energy_rel_err_mv_collision": phys.get("energy_rel_err_vs_fp64"),
            "mv_collision_chaos_floor": phys.get("chaos_floor_energy_rel"),
            "links12_value": fp32["links12"]["value"], "links12_hbm_frac": fp32["links12"]["step_hbm_frac"],
            "fp32_over_fp64": (fp32["value"] / value) if value else None}
    print(json.dumps(line), flush=True)


def batched_shapes(n_events, seed=2000):
    """Seeded uneven event sizes: transverse N in {48,64,96,128,160}, longitudinal U[2N, 3N]."""
    import numpy as np

    rng = np.random.default_rng(seed)
    shapes = []
    for _ in range(n_events):
        n = int(rng.choice([48, 64, 96, 128, 160]))
        shapes.append((n, n, int(rng.integers(2 * n, 3 * n + 1))))
    return shapes


def run_batched(args):
    """64 independent events of uneven sizes, FP32, one launch per kernel per step for all events (one
    block per tile or 128-site chunk), replayed from a CUDA graph; per-event energies reduced in FP64."""
    import torch

    from soerenpragya3dglasma_gb300 import Batch, build

    build.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    shapes = ([tuple(int(v) for v in args.event_shape.split(","))] * args.events if args.event_shape
              else batched_shapes(args.events))
    sites = sum(a * b * c for a, b, c in shapes)
    clk = ClockSampler(0)

    def timed_batch(reals, sampler=None, method="plaquette"):
        with Batch(shapes, precision="fp32", reunitarize_every=16, stream=stream) as b:
            b.set_step_method(method)
            b.set_link_reals(reals)
            for i, ev in enumerate(b.events):
                ev.fill_synthetic(2000 + i, LINK_AMP, E_AMP, J_AMP)
            tiles = b.autotune(0.1)
            b.step(0.1, max(args.warmup, 16), use_graph=True)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            if sampler is not None:
                sampler.__enter__()
            e0.record(stream)
            b.step(0.1, args.steps, use_graph=True)
            e1.record(stream)
            torch.cuda.synchronize()
            if sampler is not None:
                sampler.__exit__(None, None, None)
            return e0.elapsed_time(e1) / args.steps, b.energy(), tiles

    # the default plaquette method (each event's force summed plaquette by plaquette, 48-real
    # contributions per site)
    ms, energy, tiles = timed_batch(18, clk)
    # the same events with 12-real links (rows 0 and 1 stored; one row-2 pass per event per call)
    ms12, energy12, _ = timed_batch(12)
    # the two-pass (staple) kernels over the batch
    mst, energyt, tiles = timed_batch(18, method="two_pass")
    mst12, _, _ = timed_batch(12, method="two_pass")
    peak, peak_kind = hbm_peak()
    line = {
        "metric": "batched leapfrog site-updates/s",
        "value": sites / (ms * 1e-3),
        "unit": "site-updates/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": max(args.warmup, 16),
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (device-seeded SU(3) links / E / currents per event)",
        "config": {"workload": "%d independent events, transverse N in {48..160}, longitudinal 2N-3N, FP32, "
                               "plaquette method, reunitarise every 16, CUDA graph" % len(shapes),
                   "events": len(shapes), "sites": sites, "dt": 0.1},
        "step_hbm_frac": STEP_BYTES["fp32"] * sites / (ms * 1e-3) / 1e9 / peak,
        "peak_kind": peak_kind,
        "energy_finite": bool(all(abs(x) < float("inf") for x in energy)),
        "links12": {"value": sites / (ms12 * 1e-3), "ms_per_step": ms12,
                    "step_hbm_frac": STEP_BYTES["fp32_l12"] * sites / (ms12 * 1e-3) / 1e9 / peak,
                    "max_energy_rel_diff_vs_18_real": max(abs(x - y) / abs(y) for x, y in zip(energy12, energy))},
        "two_pass": {"value": sites / (mst * 1e-3), "ms_per_step": mst,
                     "links12_value": sites / (mst12 * 1e-3), "links12_ms_per_step": mst12,
                     "max_energy_rel_diff_vs_plaquette": max(abs(x - y) / abs(y) for x, y in zip(energyt, energy)),
                     "tiles_by_shape": sorted(set((s[0], t) for s, t in zip(shapes, tiles)))},
        "clocks": clk.summary(),
        "gpu_launches": 2 * args.steps + (args.steps // 16) * len(shapes),
    }
    print(json.dumps(line), flush=True)


def run_fft(args):
    """The gauge fixer's batched 3D FFT on its own: 8 colour planes of the lattice (default
    128x128x512, or --lattice), device to device, FP64 and FP32; GB/s counts three axis passes, each
    reading and writing the array once (the copy in and out of the work array is inside the time)."""
    import torch

    from soerenpragya3dglasma_gb300 import Lattice, build

    build.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    N = N_WORK
    vol = N[0] * N[1] * N[2]
    out = {}
    with Lattice(N, stream=stream) as lat:
        for fp32 in (False, True):
            X = torch.randn((8, N[2], N[1], N[0]), dtype=torch.complex64 if fp32 else torch.complex128, device="cuda")
            Y = torch.empty_like(X)
            for _ in range(args.warmup):
                lat.fft3d_device(X.data_ptr(), Y.data_ptr(), fp32=fp32)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                lat.fft3d_device(X.data_ptr(), Y.data_ptr(), fp32=fp32)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            out["fp32" if fp32 else "fp64"] = {"ms": ms, "gbs": 3 * 2 * (8 if fp32 else 16) * 8 * vol / (ms * 1e-3) / 1e9}
    line = {"metric": "3D FFT GB/s (8 colour planes)", "value": out["fp64"]["gbs"], "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic N(0,1)",
            "config": {"workload": "8-plane 3D FFT %dx%dx%d" % N, "lattice": list(N)}, "fp64": out["fp64"],
            "fp32": out["fp32"]}
    print(json.dumps(line), flush=True)


def run_tmd(args):
    """The TMD / Glauber initial state of SimulationmitPC::Run at the reference's parameters: 128x128x2048,
    Au nuclei (A = 197, Lorentz factor 250) centred on slices 785 and 1261, seeded noise and nucleon
    draws.  Times glasma_tmd_init end to end (noise uploads and the host profile tables included) and
    checks the state: links unitary, Gauss law."""
    import numpy as np
    import torch

    from soerenpragya3dglasma_gb300 import Lattice, build, glauber_sample

    build.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    N = tuple(int(v) for v in args.lattice.split(",")) if args.lattice else (128, 128, 2048)
    rng = np.random.Generator(np.random.PCG64(4242))
    noise = [rng.standard_normal(8 * N[0] * N[1] * N[2]) for _ in range(2)]
    uni = rng.random(400000)
    left, used = glauber_sample(197, uni)
    right, _ = glauber_sample(197, uni[used:])
    times = []
    with Lattice(N, stream=stream) as lat:
        for i in range(3):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lat.tmd_init(noise[0], noise[1], left, right, dt=0.125)
            e1.record(stream)
            torch.cuda.synchronize()
            if i > 0:
                times.append(e0.elapsed_time(e1))
        umax, _ = lat.unitarity()
        gmax, gavg = lat.gauss()
        t00 = lat.bulk()[9]
    ms = float(np.median(times))
    line = {"metric": "TMD initial state: lattice sites per second", "value": N[0] * N[1] * N[2] / (ms * 1e-3),
            "unit": "sites/s", "n_gpus": 1, "steps": len(times), "warmup": 1, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "seeded N(0,1) noise and uniform nucleon draws (numpy PCG64 seed 4242)",
            "config": {"workload": "TMD/Glauber initial state %dx%dx%d, A=197, reference parameters" % N,
                       "lattice": list(N)},
            "ms_per_init": ms, "unitarity_max": umax, "gauss_max": gmax, "gauss_avg": gavg, "t00": t00}
    print(json.dumps(line), flush=True)


def run_precision(args):
    """The precision variant: one left-moving MV nucleus (SingleSheet over all z, as
    S/LeftNucleusSimulation.cpp:357 sets it up; g^2 mu 0.5, m 0.2, sigma_z 8, centre 0.85 Nz/2 - 1),
    256x256x1024 by default, dt 0.1, 2000 steps.  Four runs from the same seeded charges: FP64 from the
    exact initial state, FP64 from its FP32-rounded copy, FP32 (reunitarised every 16 steps, FP64
    reductions) and FP32 with 12-real links from that rounded copy.  Each observable's error of the FP32
    runs is taken against the FP64 run from the same rounded start; the two FP64 runs give the floor that
    the rounding of the start alone sets (the evolution amplifies it).  Observables every
    --measure-every steps: T00, the electric and magnetic sums, the Gauss-law violation (max, avg), the
    unitarity violation and P_L/P_T of the central 32 slices (from the energy-momentum map)."""
    import numpy as np
    import torch

    from soerenpragya3dglasma_gb300 import Lattice, build

    build.build()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    N = N_WORK if args.lattice else (256, 256, 1024)
    dt, steps, every = 0.1, args.prec_steps, args.measure_every
    centre = int(0.85 * N[2] / 2 - 1)
    z0, z1 = N[2] // 2 - 16, N[2] // 2 + 16
    zeta = np.random.default_rng(1003).standard_normal(8 * N[0] * N[1])
    vol = N[0] * N[1] * N[2]

    def measure(lat):
        b = lat.bulk()
        gmax, gavg = lat.gauss()
        umax, uavg = lat.unitarity()
        r, _, _ = lat.pressure_anisotropy(z0, z1)
        # P_L = TZZ and P_T = (TXX + TYY) / 2 of the whole lattice (the central slices' ratio is
        # ill-conditioned here: the nucleus moves away from them and leaves P_T ~ 0 there)
        return {"T00": b[9], "ELECTRIC": b[13], "MAGNETIC": b[14], "P_L": b[12], "P_T": 0.5 * (b[10] + b[11]),
                "gauss_max": gmax, "gauss_avg": gavg, "unitarity_max": umax, "pl_over_pt_central": r}

    def evolve(lat):
        rows = [measure(lat)]
        ms = 0.0
        for _ in range(steps // every):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lat.step(dt, every, save_uold=True)  # UOld of the last step feeds the energy-momentum map
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
            rows.append(measure(lat))
        return rows, ms / steps

    runs, rounded = {}, {}
    t_start = time.time()
    with Lattice(N, stream=stream) as lat:
        lat.mv_init(zeta, None, qs=(0.5, 0.5), centers=(centre, centre), sigma=8.0, lam=1.65, meff=0.2, dt=dt)
        for k in INPUT_FIELDS:  # the FP32-rounded copy of the start, on the device
            buf = torch.empty(lat.field_doubles(k), dtype=torch.float64, device=dev)
            lat.download_device(k, buf.data_ptr())
            for c0 in range(0, buf.numel(), 1 << 28):
                v = buf[c0:c0 + (1 << 28)]
                v.copy_(v.to(torch.float32).to(torch.float64))
            rounded[k] = buf
        torch.cuda.synchronize()
        runs["fp64_exact_start"] = evolve(lat)
    for tag, prec, reals in (("fp64", "fp64", 18), ("fp32", "fp32", 18), ("fp32_links12", "fp32", 12)):
        with Lattice(N, precision=prec, reunitarize_every=16 if prec == "fp32" else 0, stream=stream) as lat:
            lat.link_reals = reals
            for k in INPUT_FIELDS:
                lat.upload_device(k, rounded[k].data_ptr())
            lat.upload_device("UOld", rounded["U"].data_ptr())
            torch.cuda.synchronize()
            runs[tag] = evolve(lat)
    ref = runs["fp64"][0]

    def rel(rows, name, k):
        a, b = rows[k][name], ref[k][name]
        return abs(a - b) / abs(b) if b != 0 else abs(a - b)

    names = list(ref[0].keys())
    errors = {}
    for tag in ("fp32", "fp32_links12", "fp64_exact_start"):
        rows = runs[tag][0]
        errors[tag] = {n: {"final": rel(rows, n, -1), "max_over_run": max(rel(rows, n, k) for k in range(len(rows)))}
                       for n in names}
    line = {
        "workload": "precision variant: single left-moving MV nucleus %dx%dx%d (g^2 mu 0.5, m 0.2, sigma_z 8, "
                    "centre %d), dt %g, %d steps; FP64 and FP32 (reunitarised every 16 steps) from the same "
                    "FP32-rounded start" % (N + (centre, dt, steps)),
        "ms_per_step": {t: runs[t][1] for t in runs},
        "site_updates_per_s": {t: vol / (runs[t][1] * 1e-3) for t in runs},
        "hbm_frac": {t: STEP_BYTES[{"fp64": "fp64", "fp64_exact_start": "fp64", "fp32": "fp32",
                                    "fp32_links12": "fp32_l12"}[t]] * vol / (runs[t][1] * 1e-3) / 1e9 / hbm_peak()[0]
                     for t in runs},
        "rel_error_vs_fp64_same_start": {t: errors[t] for t in ("fp32", "fp32_links12")},
        "floor_fp64_rounded_vs_exact_start": errors["fp64_exact_start"],
        "final": {t: runs[t][0][-1] for t in runs},
        "measure_every": every,
        "wall_s": time.time() - t_start,
        "note": "ms_per_step includes SaveOldLink on the last step of every %d-step call" % every,
    }
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """The adjoint workload: a 64x64x256 MV collision (g^2 mu = 0.5, m = 0.2, sigma_z = 4, centres
    128 -+ 24, seeded charges), FP64, 400 steps at dt = 0.125, objective P_L/P_T over the central 32
    slices, checkpoints every 50 steps.  Reports the adjoint's wall time (forward with checkpoints,
    then the time-reversed backward pass) over the plain forward's, and central differences
    (eps = 1e-6) along seeded random directions of E and the currents."""
    import numpy as np
    import torch

    from soerenpragya3dglasma_gb300 import Lattice, build

    build.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    N, dt, steps, every, z0, z1 = (64, 64, 256), 0.125, args.adj_steps, 50, 112, 144
    rng = np.random.default_rng(1004)
    zl, zr = rng.standard_normal(8 * N[0] * N[1]), rng.standard_normal(8 * N[0] * N[1])
    names = ("E", "Jp", "Jm", "JpStat", "JmStat")
    with Lattice(N, stream=stream) as lat:
        lat.mv_init(zl, zr, qs=(0.5, 0.5), centers=(128 - 24, 128 + 24), sigma=4.0, lam=1.65, meff=0.2, dt=dt)
        f0 = lat.download_fields()

        def restore(fields):
            lat.upload_fields(fields)
            torch.cuda.synchronize()

        def objective_after(fields):
            restore(fields)
            lat.step(dt, steps, save_uold=False)
            return lat.objective(z0, z1, Lattice.PL_OVER_PT)

        lat.step(dt, 3, save_uold=False)  # warm-up
        restore(f0)
        t0 = time.perf_counter()
        lat.step(dt, steps, save_uold=False)
        torch.cuda.synchronize()
        fwd_s = time.perf_counter() - t0
        L_fwd = lat.objective(z0, z1, Lattice.PL_OVER_PT)
        restore(f0)
        t0 = time.perf_counter()
        L_adj, _ = lat.adjoint(dt, steps, z0, z1, Lattice.PL_OVER_PT, checkpoint_every=every, grads=False)
        torch.cuda.synchronize()
        adj_s = time.perf_counter() - t0
        restore(f0)
        _, grads = lat.adjoint(dt, steps, z0, z1, Lattice.PL_OVER_PT, checkpoint_every=every)
        checks, dirs = [], []
        eps = 1e-6
        for k in range(args.fd_dirs):
            drng = np.random.default_rng(3000 + k)
            d = {}
            for name in names:
                v = drng.standard_normal(f0[name].shape)
                v[0], v[-1] = v[1], v[-2]  # ghost slices: copies of the boundary slices
                d[name] = v
            fp = dict(f0)
            fm = dict(f0)
            for name in names:
                fp[name] = f0[name] + eps * d[name]
                fm[name] = f0[name] - eps * d[name]
            fd = (objective_after(fp) - objective_after(fm)) / (2 * eps)
            ad = sum(float(np.sum(grads[name][1:-1] * d[name][1:-1])) for name in names)
            checks.append({"fd": fd, "adjoint": ad, "rel_diff": abs(fd - ad) / max(abs(fd), 1e-300)})
            dirs.append(d)
        # eps sweep along the direction with the largest difference: the central difference's truncation
        # error falls as eps^2 and its rounding error grows as ~1e-16 |L| / eps, so where the difference
        # to the adjoint is FD noise it changes with eps, and the fourth-order difference removes the
        # truncation part
        sweep = None
        if checks:
            k = max(range(len(checks)), key=lambda i: checks[i]["rel_diff"])
            d = dirs[k]

            def shifted(h):
                fs = dict(f0)
                for name in names:
                    fs[name] = f0[name] + h * d[name]
                return objective_after(fs)

            rows = []
            for e in (1e-4, 1e-5, 1e-6, 1e-7):
                fpe, fme = shifted(e), shifted(-e)
                c2 = (fpe - fme) / (2 * e)
                row = {"eps": e, "fd": c2, "rel_diff": abs(c2 - checks[k]["adjoint"]) / abs(checks[k]["adjoint"])}
                if e >= 1e-5:
                    c4 = (8 * (fpe - fme) - (shifted(2 * e) - shifted(-2 * e))) / (12 * e)
                    row.update({"fd4": c4, "rel_diff4": abs(c4 - checks[k]["adjoint"]) / abs(checks[k]["adjoint"])})
                rows.append(row)
            sweep = {"direction": k, "adjoint": checks[k]["adjoint"], "rows": rows}
    # ---- the same adjoint on an FP32 lattice (FP32 end to end), against the FP64 gradient
    with Lattice(N, precision="fp32", stream=stream) as l32:
        l32.upload_fields(f0)
        l32.step(dt, 3, save_uold=False)  # warm-up
        l32.upload_fields(f0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        l32.step(dt, steps, save_uold=False)
        torch.cuda.synchronize()
        fwd32_s = time.perf_counter() - t0
        L32_fwd = l32.objective(z0, z1, Lattice.PL_OVER_PT)
        l32.upload_fields(f0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L32, _ = l32.adjoint(dt, steps, z0, z1, Lattice.PL_OVER_PT, checkpoint_every=every, grads=False)
        torch.cuda.synchronize()
        adj32_s = time.perf_counter() - t0
        l32.upload_fields(f0)
        _, g32 = l32.adjoint(dt, steps, z0, z1, Lattice.PL_OVER_PT, checkpoint_every=every)
    rel = {name: float(np.linalg.norm(g32[name][1:-1] - grads[name][1:-1]) / np.linalg.norm(grads[name][1:-1]))
           for name in names}
    fp32 = {"forward_s": fwd32_s, "adjoint_s": adj32_s, "adjoint_over_forward": adj32_s / fwd32_s,
            "speedup_over_fp64_adjoint": adj_s / adj32_s, "objective": L32, "objective_forward": L32_fwd,
            "objective_rel_diff_vs_fp64": abs(L32 - L_adj) / abs(L_adj),
            "gradient_rel_l2_vs_fp64": rel,
            "note": "initial state rounded to FP32 on upload; the FP64 gradient is of the unrounded state"}
    line = {
        "metric": "adjoint cost: adjoint time / forward time",
        "value": adj_s / fwd_s,
        "unit": "x",
        "n_gpus": 1,
        "steps": steps,
        "warmup": 3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "MV collision from seeded N(0,1) charges (numpy PCG64 seed 1004), built on the GPU",
        "config": {"workload": "adjoint of P_L/P_T, 64x64x256 MV collision, %d steps, checkpoints every %d, "
                               "z in [%d, %d)" % (steps, every, z0, z1),
                   "lattice": list(N), "dt": dt, "g2mu": 0.5, "m": 0.2, "sigma_z": 4.0},
        "forward_s": fwd_s,
        "adjoint_s": adj_s,
        "objective": L_adj,
        "objective_forward": L_fwd,
        "fd_checks": checks,
        "fd_eps": eps,
        "fd_eps_sweep": sweep,
        "fp32": fp32,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-impl", default="auto", choices=["auto", "port", "reference"],
                    help="CPU legs: the reference's own compiled code where it was built (auto), or the oracle port")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--no-gauge", action="store_true", help="skip the gauge-fixing / FFT leg")
    ap.add_argument("--step-method", default="plaquette", choices=["one_pass", "two_pass", "plaquette", "march"])
    ap.add_argument("--fp32-step-method", default=None, choices=["one_pass", "two_pass", "plaquette", "march"],
                    help="step method of the FP32 legs (default: --step-method)")
    ap.add_argument("--march-chunk", type=int, default=0, help="z slices per block of the marching step")
    ap.add_argument("--fp64-arith", default="native", choices=["native", "double_float"],
                    help="arithmetic of the FP64 plaquette force kernel")
    ap.add_argument("--gauge-evolve", type=int, default=40, help="leapfrog steps of the MV state before gauge fixing")
    ap.add_argument("--gauge-iters", type=int, default=300, help="cap of the gauge-fixing iterations")
    ap.add_argument("--local-gauge-iters", type=int, default=20,
                    help="iterations of the Los Alamos and Jacobi gauge fixers timed on the same state")
    ap.add_argument("--only", default="both", choices=["both", "fp64", "fp32"],
                    help="which precisions to run (profiling runs); the JSON line needs both")
    ap.add_argument("--lattice", default=None, help="Nx,Ny,Nz instead of the workload's (profiling runs)")
    ap.add_argument("--event-shape", default=None, help="NX,NY,NZ for every batched event (profiling runs)")
    ap.add_argument("--prec-steps", type=int, default=2000, help="steps of the precision workload")
    ap.add_argument("--measure-every", type=int, default=100, help="measurement cadence of the precision workload")
    ap.add_argument("--workload", default="production",
                    choices=["production", "batched", "adjoint", "fft", "tmd", "precision"],
                    help="production: the headline 128x128x512 line; batched: 64 uneven events in one launch; "
                         "adjoint: the gradient of P_L/P_T on a 64x64x256 collision; fft: the 3D FFT alone; "
                         "tmd: the TMD/Glauber initial state at 128x128x2048")
    ap.add_argument("--adj-steps", type=int, default=400)
    ap.add_argument("--fd-dirs", type=int, default=2)
    ap.add_argument("--events", type=int, default=64)
    ap.add_argument("--tile", type=int, default=0, help="fixed electric-field tile width instead of autotuning")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.lattice:
        global N_WORK
        N_WORK = tuple(int(v) for v in args.lattice.split(","))
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "fft":
        run_fft(args)
    elif args.workload == "tmd":
        run_tmd(args)
    elif args.workload == "precision":
        run_precision(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

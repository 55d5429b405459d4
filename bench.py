"""Benchmark: grid-point RK4 steps per second of the trans_bl stage on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form mixed|plain]
                    [--impl ours|reference]

Workload: the 3D Blasius/TS case nx=1025, ny=193, 32 Fourier modes (P=64),
4-level multigrid, Poisson residual 1e-10 (synthetic inputs: Falkner-Skan
base flow, generated coefficient tables, seeded wall-forcing phases).
One step = one RK4 time step (four stages) over the whole domain.

value  : Mpt-steps/s = nx*ny*kfour*steps / device time, all ranks summed
         (replicas: every rank advances its own simulation; no collective).
e2e    : the same through the C ABI with the state uploaded from pinned host
         memory before and read back after every step.
The CPU baseline is the oracle (C++ restatement of the reference CPU path)
timed on one RK stage of the same workload on the host cores.
With --impl reference the whole line times that restatement instead, with
all host threads, one RK stage per sample.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Mpt-steps/s (1 GB300): batched+mixed+learned vs plain FP64 at <=1e-6 rel err"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--form", default="mixed", choices=["mixed", "plain"],
                   help="mixed: FP32 multigrid inside FP64 defect correction (default); plain: the reference's FP64 SOR")
    p.add_argument("--workload", default="config2", choices=["config2", "small"],
                   help="small: 129x65x8 grid for profiler captures")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    return p.parse_args()


def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        import torch.distributed as dist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return rank, world, dist
    return rank, world, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.samples, self.stop_ev, self.th = index, [], threading.Event(), None

    def _run(self):
        while not self.stop_ev.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self.stop_ev.wait(0.2)

    def __enter__(self):
        self.th = threading.Thread(target=self._run, daemon=True)
        self.th.start()
        return self

    def __exit__(self, *a):
        self.stop_ev.set()
        self.th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "", 1).isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 2 + i and s[2 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


WORKLOAD = {"name": "config2"}


def workload(form):
    from trans_bl_gb300 import api, configs
    prec = api.FORM_MIXED if form == "mixed" else api.FORM_PLAIN_FP64
    if WORKLOAD["name"] == "small":
        return configs.small(nx=129, ny=65, kfour=8, kphys=16, msh=3, tol=1e-10, precision=prec)
    return configs.config2(tol=1e-10, precision=prec)


def cpu_stage_sample(cfg, coefs, base, state, threads, t):
    """Time one RK stage of the oracle on the given state (seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as ora
    os.environ["OMP_NUM_THREADS"] = str(threads)
    o = ora.Oracle(cfg, coefs, base)
    if state is not None:
        o.put_state(state)
    t0 = time.perf_counter()
    o.rk_stage(1, t)
    return time.perf_counter() - t0


def run_reference(args, rank, world, dist):
    """Reference arm: the CPU restatement of the reference path, all host threads."""
    if rank != 0:
        return
    from trans_bl_gb300 import configs
    cfg = workload("plain")
    coefs, base = configs.setup_inputs(cfg)
    threads = os.cpu_count() or 1
    pts = cfg.nx * cfg.ny * cfg.kfour
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 2))
    for w in range(warm):
        cpu_stage_sample(cfg, coefs, base, None, threads, cfg.stpp + 1)
    times = [cpu_stage_sample(cfg, coefs, base, None, threads, cfg.stpp + 1) for _ in range(steps)]
    ms_per_step = 4.0 * 1e3 * float(np.mean(times))
    value = pts / (ms_per_step * 1e-3) / 1e6
    sample = "one RK stage (of four) of the nx=1025 ny=193 K=32 step from the initial state, %d samples" % steps
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mpt-steps/s", "n_gpus": world,
            "steps": steps, "warmup": warm, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "blasius_ts_3d nx=1025 ny=193 kfour=32 kphys=64 msh=4 tol=1e-10",
                       "form": "reference CPU path (C++ restatement, OpenMP over modes and lines)"},
            "cpu_baseline": {"value": value, "unit": "Mpt-steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "Mpt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    WORKLOAD["name"] = args.workload
    rank, world, dist = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, dist)
        return
    from trans_bl_gb300 import api, configs
    form = args.form
    cfg = workload(form)
    coefs, base = configs.setup_inputs(cfg)
    ctx = api.Context(cfg, coefs, base)
    pts = cfg.nx * cfg.ny * cfg.kfour
    # start from a disturbed state past the one-period forcing ramp, so every
    # mode carries a disturbance and every solve does work
    ctx.put_state(configs.disturbed_state(cfg, base, np.random.default_rng(5)))
    t = cfg.stpp + 1
    for _ in range(max(3, args.warmup)):
        ctx.step(t)
        t += 1
    ctx.synchronize()
    # timed region: device events on the library stream
    import torch
    stream_ptr = C_stream(ctx)
    ext = torch.cuda.ExternalStream(stream_ptr)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = ctx.launch_count()
    ctx.profile(True)
    barrier(dist)
    torch.cuda.synchronize()
    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ev0.record(ext)
        for _ in range(args.steps):
            ctx.step(t)
            t += 1
        ev1.record(ext)
        ev1.synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    ms = ev0.elapsed_time(ev1)
    launches = ctx.launch_count() - launches0
    sor_ms, sor_n = ctx.profile_read("sor")
    poi_ms, poi_n = ctx.profile_read("poi_uy")
    stage_ms, stage_n = ctx.profile_read("stage")
    nl_ms, nl_n = ctx.profile_read("nlterms")
    x_ms, x_n = ctx.profile_read("xlines")
    def_ms, def_n = ctx.profile_read("defect")
    r0_ms, r0_n = ctx.profile_read("relax0")
    ctx.profile(False)
    ms_max = max_over_ranks(dist, ms)
    ms_per_step = ms_max / args.steps
    value = world * pts * args.steps / (ms_max * 1e-3) / 1e6
    # roofline of the dominant kernel family
    hbm_peak, peak_kind = peaks()
    stats = ctx.poisson_stats()
    if form == "plain":
        # line-SOR: per point and sweep, read fc and sc, write fc (3 x 16 B)
        sweeps_pts = sor_points_per_launch(cfg)
        bytes_per_launch = 48.0 * sweeps_pts
        dom = {"kernel": "k_sor (lexicographic y-line SOR, one CTA per mode)", "ms": sor_ms, "launches": sor_n}
        achieved = bytes_per_launch / (sor_ms * 1e-3 / max(sor_n, 1)) / 1e9 if sor_n else 0.0
    else:
        # finest-level coloured y-line relaxation, FP32 complex (8 B): per
        # sweep (4 launches) every interior point reads r once, writes e once
        # and its e is read by the lines of the two other colours (2 x 8 B)
        bytes_per_launch = 32.0 * cfg.kfour * cfg.ny * (cfg.nx - 2) / 4.0
        dom = {"kernel": "k_relax (finest level, one warp per y-line and mode)", "ms": r0_ms, "launches": r0_n}
        achieved = bytes_per_launch / (r0_ms * 1e-3 / max(r0_n, 1)) / 1e9 if r0_n else 0.0
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "traffic": None, "peak_source": peak_kind,
            "kernel": dom["kernel"], "kernel_ms_total": dom["ms"], "kernel_launches": dom["launches"],
            "share_of_step": dom["ms"] / ms if ms > 0 else None}
    line = {"metric": METRIC, "value": value, "unit": "Mpt-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if form == "plain" else "f64+f32",
            "data": "synthetic (Falkner-Skan base flow, generated coefficients, seeded TS forcing phases)",
            "config": {"workload": "blasius_ts_3d nx=%d ny=%d kfour=%d kphys=%d msh=%d tol=1e-10 steps_per_period=%d" % (
                           cfg.nx, cfg.ny, cfg.kfour, cfg.kphys, cfg.msh, cfg.stpp),
                       "form": form, "replicas": world, "l2": "working set ~4 GB > L2 (129 MB)",
                       "start": "disturbed state (1e-3) past the forcing ramp",
                       "iterations_per_mode_last_solve": float(np.mean(stats["vcycles"][:cfg.kfour]))},
            "roofline": roof, "gpu_launches": launches,
            "breakdown_ms": {"stage": stage_ms, "poi_uy": poi_ms, "relax_sweeps": sor_ms, "relax_finest": r0_ms,
                             "fp64_defect": def_ms, "nlterms": nl_ms, "xlines": x_ms},
            "clocks": clk.summary()}
    if not args.no_e2e:
        line["e2e"] = e2e_measure(ctx, cfg, t, max(1, min(args.steps, 3)), world, dist)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        st = ctx.get_state()
        cpu_s = cpu_stage_sample(cfg, coefs, base, st, 1, t)
        cpu_val = pts / (4.0 * cpu_s) / 1e6
        line["cpu_baseline"] = {"value": cpu_val, "unit": "Mpt-steps/s", "cores": 1, "kind": "port",
                                "sample": "one RK stage of the same nx=1025 ny=193 K=32 state, single thread "
                                          "(%.1f s); per-step rate = stage rate / 4" % cpu_s}
    if rank == 0:
        print(json.dumps(line), flush=True)


def C_stream(ctx):
    import ctypes as C
    p = C.c_void_p()
    ctx.lib.tb_stream(ctx.h, C.byref(p))
    return p.value or 0


def sor_points_per_launch(cfg):
    """Average point-sweeps per k_sor launch of one V-cycle (all modes)."""
    nx, ny, msh, K = cfg.nx, cfg.ny, cfg.msh, cfg.kfour
    lv = []
    px, py = nx, ny
    for _ in range(msh):
        lv.append((px, py))
        px, py = (px + 1) // 2, (py + 1) // 2
    launches, pts = 0, 0
    for l in range(msh - 1):
        launches += 2
        pts += (3 + 1) * (lv[l][0] - 2) * lv[l][1]
    launches += 1
    pts += 60 * (lv[-1][0] - 2) * lv[-1][1]
    return K * pts / launches


def e2e_measure(ctx, cfg, t, steps, world, dist):
    """Steps through the C ABI with pinned host buffers copied in and out each step."""
    import torch
    shape = (cfg.kfour, cfg.ny, cfg.nx)
    host = {n: torch.empty(shape + (2,), dtype=torch.float64, pin_memory=True)
            for n in ("ux", "uy", "uz", "wx", "wy", "wz")}
    st = ctx.get_state()
    for n, v in st.items():
        host[n].numpy()[...] = np.stack([v.real, v.imag], axis=-1)
    import ctypes as C
    D = C.POINTER(C.c_double)
    ptrs = [C.cast(host[n].data_ptr(), D) for n in ("ux", "uy", "uz", "wx", "wy", "wz")]
    nbytes = sum(h.numel() * 8 for h in host.values())
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(steps):
        api_check(ctx.lib.tb_put_state(ctx.h, *ptrs))
        api_check(ctx.lib.tb_step(ctx.h, t))
        api_check(ctx.lib.tb_get_state(ctx.h, *ptrs))
        t += 1
    el = time.perf_counter() - t0
    el = max_over_ranks(dist, el)
    pts = cfg.nx * cfg.ny * cfg.kfour
    return {"value": world * pts * steps / el / 1e6, "unit": "Mpt-steps/s", "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes, "steps": steps}


def api_check(rc):
    from trans_bl_gb300 import api
    api.check(rc, "e2e")


if __name__ == "__main__":
    main()

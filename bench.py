"""Benchmark of the FIM horizontal dynamics step on GB300.

Workload (default): glvl 8 (655,362 cells), nvl 64, 20 tracers + theta,
dt 45 s (FIM's glvl-8 step; 72 s exceeds the scheme's stability limit),
FP32-mixed, seeded synthetic balanced state; one "step" is one
fused dyn_run iteration (hybgen + dffusn_lev and hystat of the previous step,
abstart, edgvar1, edgvar3, cnuity, trcadv, momtum, globsum) replayed as one
CUDA graph.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  value = cell-level-steps/s of all ranks
(replicas: one independent state per GPU), timed with CUDA events on the
library's stream, max over ranks.  The state (~60 GB) is far larger than L2,
so no flush is needed between steps.  The reference arm times the CPU oracle
(the C restatement of the reference's Fortran routines) on a level-6 sample
of the same workload with all host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

METRIC = "cell-level-steps/s at glvl 8 nvl 64, FP32-mixed vs FP64; served p50/p99 latency"
UNIT = "cell-level-steps/s"

# Algorithmic words per cell-level per step that each kernel must read and
# write once (own-column values; neighbour values are re-reads served by
# L1/L2), summed over the tracers it handles.  Used for roofline.achieved.
WORDS = {
    # the fused step averages only the layer thickness in edgvar3; the
    # tracers' edge values are formed on chip by k_trf_lo/k_trf_hi
    "k_edgvar1": lambda T: 41, "k_edgvar3_own": lambda T: 7, "k_edgvar3_avg": lambda T: 12,
    # edgvar2 (hiOrderUVComp): speeds and gradient (u, v, 6+6 edge winds in,
    # 3 out), then the correction (3 + 12 in, 18 out)
    "k_edgvar2_grad": lambda T: 17, "k_edgvar2": lambda T: 33,
    # tracer transport on cell patches: per tracer, k_trf_lo reads the tracer,
    # tracer x thickness and two low-order AB3 slots and writes one slot,
    # trcr_lo, S+, S-, the old tracer's copy and six antidiffusive fluxes
    # (15), and reads the mass fluxes (6), the thickness and theta's six edge
    # values (13); k_trf_hi reads the copy, trcr_lo, S+, S-, two AB3 slots,
    # the six fluxes, the low-order tendency and tracer x thickness and writes
    # one slot, tracer x thickness and the tracer (17), and reads the
    # thickness (1)
    "k_trf_lo": lambda T: 15 * T + 13, "k_trf_hi": lambda T: 17 * T + 1,
    "k_cnuity12": lambda T: 37, "k_cnuity3": lambda T: 8, "k_cnuity4": lambda T: 26, "k_cnuity5": lambda T: 14,
    # cnuity1..4 as one persistent launch (--persistent): the three kernels' words
    "k_cnuity_coop": lambda T: 37 + 8 + 26,
    "k_trcadv1": lambda T: 27 * T, "k_trcadv2": lambda T: 16 * T, "k_trcadv3": lambda T: 18 * T,
    "k_dissip": lambda T: 5, "k_del4prep": lambda T: 4, "k_momtum1": lambda T: 44,
    # in the step the remap also writes tracer x thickness (T words), which
    # k_hystat_trdp then leaves out
    "k_regrid": lambda T: 3, "k_dffusn_lev": lambda T: 2, "k_remap": lambda T: 3 * T + 10, "k_inflate": lambda T: 2,
    "k_hystat": lambda T: 7, "k_hystat_trdp": lambda T: 2 * T + 3, "k_globsum_levels": lambda T: T + 1,
}

E2E_FIELDS = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "trdp", "u_tdcy", "v_tdcy",
              "dp_tdcy", "dpl_tdcy", "trc_tdcy", "trl_tdcy", "ws3d", "sdot", "relvor", "psrf", "ptdcy"]
# AB3 tendency fields (a step reads slots of and vof and writes slot nf) and
# the fields a step writes without reading them
E2E_AB3 = {"u_tdcy", "v_tdcy", "dp_tdcy", "dpl_tdcy", "trc_tdcy", "trl_tdcy"}
E2E_OUTPUTS = {"ws3d", "sdot", "relvor"}  # rewritten whole by every step (ptdcy: one of its two levels)
# rewritten whole by the step's opening hybgen and hystat from a member's
# second step on (the timed steps): they only come down
E2E_RECOMPUTED = {"mp3d", "trdp", "dp3d"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                self.out = ""

    def summary(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm, mx, reasons = [], [], set()
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws, backend_device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=backend_device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------------ GPU arm --
def make_state(F, grid, cfg, wl, dtype):
    dyc = F.Dycore(grid, cfg)
    st = dyc.state()
    for m in range(cfg.members):
        fields = F.synthetic_state(grid, cfg, seed=wl["seed"] + m, sigma_ps=wl["sigma_ps"], noise=wl["noise"],
                                   dtype=dtype)
        st.load(fields, member=m)
        del fields
    st.init()
    return dyc, st


def timed_steps(torch, dyc, st, k, graph=True):
    stream = torch.cuda.ExternalStream(dyc.stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    n0 = dyc.launches()
    a.record(stream)
    for _ in range(k):
        st.step(use_graph=graph)
    b.record(stream)
    b.synchronize()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / k, dyc.launches() - n0


def gpu_arm(args, ws, rank, local):
    import torch
    import fimocn_subx_realtime_hera_apr2020_gb300 as F

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl = dict(F.WORKLOADS[args.workload])
    members = args.members or wl.get("members", 1)
    grid = F.Grid.cached(wl["glvl"])
    N, L, T = grid.nip, wl["nvl"], wl["ntra"]
    units = N * L * members  # cell-levels per step per GPU
    group = args.member_group if args.member_group >= 0 else wl.get("member_group", 0)
    cfg = F.FimConfig(nvl=L, ntra=T, dt=wl["dt"], precision="f32", members=members, member_group=group,
                      hi_order_uv_comp=1 if args.hi_order_uv else 0)
    dyc, st = make_state(F, grid, cfg, wl, np.float32)
    if args.persistent:
        dyc.set_persistent(True)
    for _ in range(args.warmup):
        st.step(use_graph=True)
    torch.cuda.synchronize()
    barrier(ws)
    with Clocks(local) as clk:
        ms, launches = timed_steps(torch, dyc, st, args.steps, graph=True)
    barrier(ws)
    ms_max = max_over_ranks(ms, ws, torch.device("cuda", local))
    value = units * ws / (ms_max * 1e-3)
    rc, flags = st.check()
    if rc != 0:
        raise SystemExit("device status flags %d after the timed steps" % flags)
    shape = dyc.tracer_shape()

    # per-kernel times (events on the library stream), direct launches
    dyc.profile(True)
    kp = max(2, min(args.steps, 5))
    for _ in range(kp):
        st.step(use_graph=False)
    torch.cuda.synchronize()
    prof = dyc.profile_report()
    dyc.profile(False)
    peak, peak_kind = peaks()
    w = 4
    total = sum(v[1] for v in prof.values())
    kernels = {}
    for name, (n, tms) in prof.items():
        if name not in WORDS:
            continue
        bytes_launch = WORDS[name](T) * w * N * L * members * kp / n
        avg = tms / n
        kernels[name] = {"launches": n, "ms_total": tms, "share": tms / total, "ms_avg": avg,
                         "alg_bytes": bytes_launch, "gbs": bytes_launch / (avg * 1e-3) / 1e9}
    dom = max(kernels, key=lambda k: kernels[k]["ms_total"])
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get(args.workload, {}).get(dom)
        except Exception:
            traffic = None
    roof = {"bound": "hbm", "kernel": dom, "achieved": kernels[dom]["gbs"], "peak": peak, "unit": "GB/s",
            "frac": kernels[dom]["gbs"] / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic, "alg_bytes_per_launch": kernels[dom]["alg_bytes"]}
    # the whole step against its compulsory traffic: every state word read and
    # written once (29 + 10 ntra words per cell-level) plus the grid tables
    # read once (118 FP32 metric values and 49 int32 index values per cell)
    step_bytes = (29 + 10 * T) * w * N * L * members + (118 * w + 49 * 4) * N
    roof["step"] = {"compulsory_bytes": step_bytes, "ms_per_step": ms_max,
                    "achieved": step_bytes / (ms_max * 1e-3) / 1e9, "unit": "GB/s",
                    "frac": step_bytes / (ms_max * 1e-3) / 1e9 / peak,
                    "kernel_words_per_cell_level": sum(WORDS[k](T) for k in kernels),
                    "compulsory_words_per_cell_level": 29 + 10 * T}

    # end to end through the C-ABI with host buffers: every step uploads what it
    # reads and downloads what it writes (AB3 tendency fields: the two slots it
    # reads, the one it writes; omega, sdot and relvor are outputs only, and so
    # are the Montgomery potential and tracer x thickness at the timed steps)
    e2e = None
    if not args.no_e2e:
        bufs = {}
        for f in E2E_FIELDS:
            ptr, n = st.field_ptr(f, 0)
            bufs[f] = torch.empty(n * members, dtype=torch.float32, pin_memory=True)
            for m in range(members):
                st.download(f, m, out=bufs[f][m * n:(m + 1) * n].numpy())
        lib, ctx, sst, fid = dyc.lib, dyc.ctx, st.st, F.dycore._lib.FIELD_ID

        def one_step():
            h2d = d2h = 0
            slots = [st.next_slots(m) for m in range(members)]
            for f, buf in bufs.items():
                if f in E2E_OUTPUTS or f in E2E_RECOMPUTED:
                    continue
                n = buf.numel() // members
                for m in range(members):
                    hp = buf.data_ptr() + m * n * 4
                    if f in E2E_AB3:
                        for sl in slots[m][1:]:
                            _check(lib.fim_state_upload_slot(ctx, sst, fid[f], m, sl, hp), "upload slot")
                        h2d += 2 * n // 3 * 4
                    else:
                        _check(lib.fim_state_upload(ctx, sst, fid[f], m, hp), "upload")
                        h2d += n * 4
            st.step(use_graph=True)
            for f, buf in bufs.items():
                n = buf.numel() // members
                for m in range(members):
                    hp = buf.data_ptr() + m * n * 4
                    if f in E2E_AB3:
                        _check(lib.fim_state_download_slot(ctx, sst, fid[f], m, slots[m][0], hp), "download slot")
                        d2h += n // 3 * 4
                    else:
                        _check(lib.fim_state_download(ctx, sst, fid[f], m, hp), "download")
                        d2h += n * 4
            return h2d, d2h

        stream = torch.cuda.ExternalStream(dyc.stream)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ke = max(1, min(args.steps, 5))

        def timed(fn):
            torch.cuda.synchronize()
            a.record(stream)
            for _ in range(ke):
                moved = fn()
            b.record(stream)
            b.synchronize()
            return max_over_ranks(a.elapsed_time(b) / ke, ws, torch.device("cuda", local)), moved

        # the library's step with host transfers: the registered pinned
        # buffers go up stage by stage as the step needs them and come down as
        # soon as their last writer is done, beside the kernels
        for f, buf in bufs.items():
            n = buf.numel() // members
            for m in range(members):
                st.set_host(f, buf[m * n:(m + 1) * n], m)
        # warm-up steps first: the first copies out of freshly pinned host
        # buffers take far longer (~0.2 s at glvl 8) than every later one
        for _ in range(max(1, args.warmup)):
            st.step_io()
        e_ms, (h2d, d2h) = timed(st.step_io)
        # the same transfers issued one after the other around a resident step
        for _ in range(max(1, args.warmup)):
            one_step()
        s_ms, (sh2d, sd2h) = timed(one_step)
        assert (sh2d, sd2h) == (h2d, d2h), ((sh2d, sd2h), (h2d, d2h))
        # one more step with the library's timeline marks (outside the timed
        # steps): when each stage's uploads end, its kernels are done and its
        # downloads end, in ms from the step's start
        dyc.profile(True)
        st.step_io()
        torch.cuda.synchronize()
        tl = {k[3:]: v[1] / v[0] for k, v in dyc.profile_report().items() if k.startswith("io:")}
        dyc.profile(False)
        tl_keys = [k for k in tl if k.startswith(("up_end", "computed", "down_end"))] + ["end"]
        timeline = {k: round(tl[k], 2) for k in sorted(tl_keys, key=lambda k: tl[k]) if k in tl}
        # the same path for a driver that leaves the dynamics' own AB3
        # tendency history on the device (not registered: the step reads and
        # writes the device slots, which hold the current values)
        for f in E2E_AB3:
            for m in range(members):
                st.set_host(f, None, m)
        st.step_io()
        r_ms, (rh2d, rd2h) = timed(st.step_io)
        resident = {"value": units * ws / (r_ms * 1e-3), "unit": UNIT, "ms_per_step": r_ms,
                    "h2d_bytes_per_step": rh2d, "d2h_bytes_per_step": rd2h,
                    "path": "fim_step_io with the six AB3 tendency fields left on the device"}
        e2e = {"value": units * ws / (e_ms * 1e-3), "unit": UNIT, "ms_per_step": e_ms,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "path": "fim_state_set_host (pinned host buffers) + fim_step_io: the fields the step reads go up "
                       "before the stage that first needs them, the fields it writes come down as soon as "
                       "they are final, on two copy streams beside the kernels",
               "serial_ms_per_step": s_ms, "timeline_ms": timeline, "tendencies_on_device": resident,
               "serial_path": "fim_state_upload(_slot) -> fim_step -> fim_state_download(_slot), one after the "
                              "other"}
        del bufs
    qtrcr, bud = st.budget()
    st.free()
    dyc.close()
    torch.cuda.synchronize()

    # plain FP64 GPU step at the same workload
    fp64 = None
    if args.fp64_steps > 0:
        cfg64 = F.FimConfig(nvl=L, ntra=T, dt=wl["dt"], precision="f64", members=members, member_group=group)
        d64, s64 = make_state(F, grid, cfg64, wl, np.float64)
        s64.step(use_graph=True)
        ms64, _ = timed_steps(torch, d64, s64, args.fp64_steps, graph=True)
        ms64 = max_over_ranks(ms64, ws, torch.device("cuda", local))
        fp64 = {"value": units * ws / (ms64 * 1e-3), "ms_per_step": ms64, "steps": args.fp64_steps,
                "fp32_mixed_speedup": ms64 / ms_max}
        s64.free()
        d64.close()

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(args, threads_all=True)

    # the served half of the metric: the default request stream, FP32-mixed
    served = None
    if ws == 1 and not args.no_serve:
        n = args.serve or 40
        served = {"requests": n, "rate_per_s": args.serve_rate, "slots_per_pool": args.serve_slots,
                  "glvl": [5, 6, 7], "nvl": [38, 64], "tracers": [4, 20],
                  "steps": [args.serve_min_steps, args.serve_max_steps], "precision": "fp32-mixed",
                  **serve_stats(args, n, "f32")}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (float-float column sums, FP64 budget reductions)",
            "data": "synthetic seeded balanced state (no dataset: the reference's GFS initial state is not "
                    "in the tree)",
            "config": {"workload": args.workload + ("+edgvar2" if args.hi_order_uv else "") +
                                   ("+persistent-cnuity" if args.persistent else ""), "glvl": wl["glvl"],
                       "nip": N, "nvl": L, "ntra": T,
                       "dt": wl["dt"], "members_per_gpu": members, "member_group": group or members,
                       "tracer_shape_autotuned": {"levels_per_thread": shape[0], "threads_per_block": shape[1],
                                                  "probe_ms": shape[2]},
                       "precision": "fp32-mixed",
                       "cuda_graph": True, "parallelism": "replicas" if ws > 1 else "single",
                       "l2": "no flush: state and edge fields (~60 GB) far exceed the 129 MB L2"},
            "gpu_launches": launches, "clocks": clk.summary(), "roofline": roof, "e2e": e2e,
            "cpu_baseline": cpu, "fp64": fp64, "serve": served, "kernels": kernels,
            "budget": {"qmass": bud["qmass"], "qtrcr_theta": qtrcr[0]}}
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed with status %d" % (what, rc))


# -------------------------------------------------------------- CPU oracle --
def oracle_rate(glvl, L, T, dt, steps, threads, seed=3000):
    import oracle as orc
    import fimocn_subx_realtime_hera_apr2020_gb300 as F
    from helpers import oracle_for

    orc.set_threads(threads)
    grid = F.Grid.cached(glvl)
    cfg = F.FimConfig(nvl=L, ntra=T, dt=dt)
    fields = F.synthetic_state(grid, cfg, seed=seed, sigma_ps=200.0, noise=0.0)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    o.step(s, 1)  # warm-up
    t0 = time.perf_counter()
    for its in range(2, 2 + steps):
        o.step(s, its)
    dt_s = (time.perf_counter() - t0) / steps
    return grid.nip * L / dt_s, dt_s


def cpu_baseline(args, threads_all=True):
    cores = os.cpu_count() or 1
    L, T = 64, 21
    v_all, s_all = oracle_rate(6, L, T, 180.0, 2, cores)
    v_one, s_one = oracle_rate(5, L, T, 360.0, 1, 1)
    return {"value": v_all, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "CPU oracle (C restatement of the reference Fortran routines, OpenMP) on glvl 6 "
                      "(40,962 cells), nvl 64, 21 tracers: 2 steps after 1 warm-up, %.2f s/step" % s_all,
            "value_1thread": v_one,
            "sample_1thread": "glvl 5 (10,242 cells), nvl 64, 21 tracers, 1 step, %.2f s/step" % s_one}


def reference_arm(args, ws, rank):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    import oracle as orc
    import fimocn_subx_realtime_hera_apr2020_gb300 as F
    from helpers import oracle_for

    orc.set_threads(cores)
    glvl, L, T = 6, 64, 21
    grid = F.Grid.cached(glvl)
    cfg = F.FimConfig(nvl=L, ntra=T, dt=180.0)  # glvl-6 step, same Courant number as glvl 8 at 45 s
    fields = F.synthetic_state(grid, cfg, seed=3000, sigma_ps=200.0, noise=0.0)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    its = 0
    for _ in range(args.warmup):
        its += 1
        o.step(s, its)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        its += 1
        o.step(s, its)
    sec = (time.perf_counter() - t0) / args.steps
    value = grid.nip * L / sec
    sample = ("CPU oracle (C restatement of the reference Fortran dycore routines, OpenMP, %d threads) on a "
              "glvl-6 sample (40,962 cells) of the glvl-8 workload: nvl 64, 21 tracers, dt 180 s (the glvl-8 "
              "Courant number at 45 s), seed 3000, no wind noise; rates per cell-level compare with the GPU "
              "arm's glvl-8 run; grid tables from this project's builder (the reference's numbering and "
              "neighbour order, bit for bit), no GPU work" % cores)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic seeded balanced state",
            "config": {"workload": args.workload, "sample_glvl": glvl, "nip": grid.nip, "nvl": L, "ntra": T},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def serve_stats(args, n, prec):
    """p50/p99 latency and aggregate throughput of n served requests (the
    seeded Poisson stream), arrivals replayed in real time."""
    from fimocn_subx_realtime_hera_apr2020_gb300.serve import Server, latency_stats, poisson_requests
    reqs = poisson_requests(n, rate=args.serve_rate, seed=5000, steps=(args.serve_min_steps, args.serve_max_steps))
    srv = Server(precision=prec, slots=args.serve_slots, collect=(), grids=(5, 6, 7))
    done = srv.run(reqs, realtime=True)
    pools = {"glvl%d_nvl%d" % k: len(p.slots) for k, p in sorted(srv.pools.items())}
    srv.close()
    return {**latency_stats(done), "pool_slots": pools}


def serve_arm(args, ws, rank, local):
    """Served forecast-advance requests: a seeded Poisson stream of the mixed
    glvl 5/6/7, nvl 38/64, 4-20 tracer workload, continuous batching."""
    import torch

    torch.cuda.set_device(local)
    out = {}
    for prec in ("f32", "f64") if args.serve_fp64 else ("f32",):
        out[prec] = serve_stats(args, args.serve, prec)
    line = {"metric": "served forecast-advance latency (p50/p99) and aggregate cell-level-steps/s",
            "value": out["f32"]["p50_s"], "unit": "s", "higher_is_better": False,
            "config": {"requests": args.serve, "rate_per_s": args.serve_rate, "slots_per_pool": args.serve_slots,
                       "glvl": [5, 6, 7], "nvl": [38, 64], "tracers": [4, 20],
                       "steps": [args.serve_min_steps, args.serve_max_steps]},
            "serve": out}
    if rank == 0:
        print(json.dumps(line))


ACC_FIELDS = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "trdp"]


def accuracy_arm(args, ws, rank, local):
    """Error of the GPU paths after 1..K steps on one seeded state.

    Reference: the FP64 CPU oracle (workloads up to glvl 6), or the FP64 GPU
    path (glvl 8, where the oracle would take hours).  Per field: relative L2
    and max |error|; global mass drift (qmass / qmass(step 0) - 1) and the
    minimum over tracers 2..ntra of each run."""
    import torch
    import fimocn_subx_realtime_hera_apr2020_gb300 as F

    if rank != 0:
        return
    torch.cuda.set_device(local)
    wl = F.WORKLOADS[args.workload]
    glvl, L, T = wl["glvl"], args.nvl or 64, wl["ntra"]
    if args.workload.startswith("glvl4"):
        L = 38
    grid = F.Grid.cached(glvl)
    N = grid.nip
    K = args.accuracy
    marks = sorted({m for m in (1, 10, 50, 100, K) if m <= K})
    use_oracle = glvl <= 6
    dt = args.dt or wl["dt"]
    mk = lambda prec: F.FimConfig(nvl=L, ntra=T, dt=dt, precision=prec)  # noqa: E731
    host = F.synthetic_state(grid, mk("f64"), seed=wl["seed"], sigma_ps=wl["sigma_ps"], noise=wl["noise"])
    runs = {}
    for prec in ("f64", "f32"):
        d = F.Dycore(grid, mk(prec))
        st = d.state()
        # the FP64 fields as given: an FP32-mixed state keeps them for its
        # FP64 initial adjustment (fim_state_upload_f64)
        st.load(host)
        st.init()
        runs[prec] = (d, st)
    ref = None
    if use_oracle:
        import oracle as orc
        from helpers import oracle_for
        orc.set_threads(os.cpu_count() or 1)
        o = oracle_for(grid, mk("f64"))
        s = o.init_state(o.new_state(host))

    def fields_of(prec):
        st = runs[prec][1]
        return {n: st.tensor(n).double() for n in ACC_FIELDS}

    def tracer_min(tr):
        return float(tr.reshape(T, N, L)[1:].min())

    out = {}
    qstart = {}
    for its in range(1, K + 1):
        for prec in ("f64", "f32"):
            runs[prec][1].step(its, use_graph=True)
        if use_oracle:
            qo = o.step(s, its)[1]["qmass"]
        if its == 1:
            for prec in ("f64", "f32"):
                qstart[prec] = runs[prec][1].budget()[1]["qmass"]
            if use_oracle:
                qstart["oracle"] = qo
        if its not in marks:
            continue
        torch.cuda.synchronize()
        g64, g32 = fields_of("f64"), fields_of("f32")
        refs = {n: torch.from_numpy(s[n]).cuda() for n in ACC_FIELDS} if use_oracle else g64
        rec = {}
        for name, got in (("gpu_f64", g64), ("gpu_f32", g32)):
            if name == "gpu_f64" and not use_oracle:
                continue
            per = {}
            for n in ACC_FIELDS:
                d = got[n] - refs[n]
                per[n] = {"rel_l2": float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(refs[n])),
                          "max_abs": float(d.abs().max())}
            rec[name] = per
        mass = {}
        for prec in ("f64", "f32"):
            mass["gpu_" + prec] = runs[prec][1].budget()[1]["qmass"] / qstart[prec] - 1
        if use_oracle:
            mass["oracle"] = qo / qstart["oracle"] - 1
        trmin = {"gpu_f64": tracer_min(g64["tr3d"]), "gpu_f32": tracer_min(g32["tr3d"])}
        if use_oracle:
            trmin["oracle"] = float(s["tr3d"].reshape(T, N, L)[1:].min())
        rec["mass_drift_since_step1"] = mass
        rec["tracer_min"] = trmin
        out[str(its)] = rec
        del g64, g32, refs
    line = {"metric": "error after K steps against the %s" % ("FP64 CPU oracle" if use_oracle else "FP64 GPU path"),
            "config": {"workload": args.workload, "glvl": glvl, "nip": N, "nvl": L, "ntra": T, "dt": dt,
                       "steps": K, "reference": "oracle" if use_oracle else "gpu_f64"},
            "checkpoints": out}
    print(json.dumps(line))
    for d, st in runs.values():
        st.free()
        d.close()


def cpl_arm(args, ws, rank, local):
    """Physics coupling (fim_cpl_dyn_to_phy / fim_cpl_phy_to_dyn, the default
    addtend = 0 path) on the workload's FP32-mixed state through the C-ABI with
    device pointers; CUDA events on the library stream around K calls each."""
    import ctypes
    import torch
    import fimocn_subx_realtime_hera_apr2020_gb300 as F

    torch.cuda.set_device(local)
    wl = dict(F.WORKLOADS[args.workload])
    grid = F.Grid.cached(wl["glvl"])
    N, L, T = grid.nip, wl["nvl"], wl["ntra"]
    NL = N * L
    cfg = F.FimConfig(nvl=L, ntra=T, dt=wl["dt"], precision="f32")
    dyc, st = make_state(F, grid, cfg, wl, np.float32)
    fp = {n: st.field_ptr(n)[0] for n in ("pr3d", "us3d", "vs3d", "ws3d", "tr3d", "dp3d")}
    gfs = {n: torch.zeros(N if n == "ps" else NL, dtype=torch.float64, device="cuda") for n in F.Dycore.GFS_NAMES}
    col = {n: torch.zeros(N, dtype=torch.float64, device="cuda") for n in ("geshem", "rainc", "evap")}
    c2d = {n: torch.zeros(N, dtype=torch.float32, device="cuda") for n in ("rn2d", "rc2d", "qf2d")}
    # without physics in between, cpl_phy_to_dyn writes back the state cpl_dyn_to_phy read
    lib, ctx = dyc.lib, dyc.ctx
    torch.cuda.synchronize()

    def d2p():
        _check(lib.fim_cpl_dyn_to_phy_r4(ctx, 1, 1, fp["pr3d"], fp["us3d"], fp["vs3d"], fp["ws3d"], fp["tr3d"],
                                         *[gfs[n].data_ptr() for n in F.Dycore.GFS_NAMES]), "cpl_dyn_to_phy")

    def p2d():
        _check(lib.fim_cpl_phy_to_dyn_r4(ctx, 1, 1, 0, 0, ctypes.c_double(wl["dt"]),
                                         *[gfs[n].data_ptr() for n in ("p", "u", "v", "q", "cld", "oz", "t")],
                                         *[col[n].data_ptr() for n in ("geshem", "rainc", "evap")], fp["dp3d"],
                                         fp["us3d"], fp["vs3d"], fp["tr3d"],
                                         *[c2d[n].data_ptr() for n in ("rn2d", "rc2d", "qf2d")]), "cpl_phy_to_dyn")

    stream = torch.cuda.ExternalStream(dyc.stream)
    res = {}
    for name, fn, nbytes in (("cpl_dyn_to_phy", d2p, (8 * 4 + 15 * 8) * NL), ("cpl_phy_to_dyn", p2d, (7 * 8 + 6 * 4) * NL)):
        for _ in range(args.warmup):
            fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        for _ in range(args.steps):
            fn()
        b.record(stream)
        b.synchronize()
        ms = a.elapsed_time(b) / args.steps
        peak, kind = peaks()
        gbs = nbytes / (ms * 1e-3) / 1e9
        res[name] = {"ms": ms, "alg_bytes": nbytes, "gbs": gbs, "frac_of_hbm": gbs / peak, "peak_source": kind}
    if rank == 0:
        print(json.dumps({"metric": "physics coupling (cpl_run) GB/s", "config": {"workload": args.workload,
                          "glvl": wl["glvl"], "nip": N, "nvl": L, "ntra": T, "precision": "fp32-mixed"},
                          "steps": args.steps, "warmup": args.warmup, "coupling": res}))
    st.free()
    dyc.close()


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="glvl8_nvl64_t20")
    p.add_argument("--members", type=int, default=0)
    p.add_argument("--member-group", type=int, default=-1, help="members per dynamics group (default: workload's)")
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--serve", type=int, default=0, help="run the serving benchmark with this many requests")
    p.add_argument("--serve-rate", type=float, default=20.0)
    p.add_argument("--serve-slots", type=int, default=8)
    p.add_argument("--serve-min-steps", type=int, default=24)
    p.add_argument("--serve-max-steps", type=int, default=240)
    p.add_argument("--serve-fp64", action="store_true")
    p.add_argument("--no-serve", action="store_true", help="leave the served stream out of the default line")
    p.add_argument("--accuracy", type=int, default=0, help="report the error after this many steps")
    p.add_argument("--nvl", type=int, default=0)
    p.add_argument("--dt", type=float, default=0.0, help="time step of the accuracy run (default: workload's)")
    p.add_argument("--cpl", action="store_true", help="time the physics coupling on the workload's state")
    p.add_argument("--hi-order-uv", action="store_true", help="the step with edgvar2 (hiOrderUVComp)")
    p.add_argument("--persistent", action="store_true", help="cnuity1..4 as one cooperative persistent launch")
    args = p.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, ws, rank)
        return
    if args.serve:
        serve_arm(args, ws, rank, local)
        return
    if args.accuracy:
        accuracy_arm(args, ws, rank, local)
        return
    if args.cpl:
        cpl_arm(args, ws, rank, local)
        return
    gpu_arm(args, ws, rank, local)


if __name__ == "__main__":
    main()

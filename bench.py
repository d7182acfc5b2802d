"""Benchmark: batched conservative regridding on one GB300.

Workload (the largest single-GPU configuration): HEALPix nside=256 (786,432
pixels, 4 great-circle corners each, nested order) <-> 0.25-degree lon-lat
(1440 x 720 = 1,036,800 cells).  R = Regridder(dst=HEALPix, src=lon-lat) is
built in FP64 on the GPU; one step applies 128 FP32 fields (8 variables x 16
levels of smooth degree-64 spherical harmonics + N(0, 0.1) noise) forward with
R and back with transpose(R).  Inputs (0.9 GB per direction) exceed the
129 MB L2, so no flush is needed between steps.

value  = algorithmic bytes of one step / device time of one step (GB/s), with
         bytes per direction = nnz*(4 col + 4 weight) + 4*(rows+1)
                               + 4*K*(cols + rows)   (each field element once).
         The reference arm divides the same byte count by its own time for
         the same 128-field step, so the two values are a time ratio.
e2e    = the same metric through the public API with pinned host buffers:
         host->device copy, SpMM, device->host copy inside the timed region.
Also reported: build pairs/s with a roofline of the clip kernel against the
FP64 peak measured by our own FMA-loop kernel, the plain FP64 apply (one
field per launch, and all 128 fields in one launch), the BF16 apply, the FP32
error against the FP64 apply, the ncu-free roofline of the SpMM kernel, the
smaller configurations (small FP64, batches, derivatives), and the CPU oracle
on the host cores.

--impl reference times the CPU restatement of the reference's regrid! (one
CSC mul! per field on Float32 fields with the Float64 matrix, fields spread
over all host threads) on the same 128-field step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "conservativeregridding.jl_gb300"))

METRIC = "build pairs/s; batched-apply GB/s & fields/s vs plain FP64 apply, 1 GB300"
WORKLOAD = "healpix256_nested <-> lonlat_0.25deg, 128 fp32 fields, R then transpose(R)"
VALUE_DEF = ("algorithmic bytes of the 128-field FP32 step (4-byte weights and columns, each field element once) "
             "/ time per step; both arms divide the same bytes")

# FP64 FLOPs of the per-pair clip + area of two quadrilaterals, a model of the
# algorithm (one-pass Sutherland-Hodgman with great-circle half-spaces, then
# the Van Oosterom-Strackee fan), not a count of the kernel's instructions:
#   side values n.(v - a):      4 clip edges x 4 subject vertices x 8 (3 sub, 3 mul, 2 add)  = 128
#   crossing points:            2 cutting stages x 2 points x 19
#                               (|s_b| a + |s_a| b: 9; dot 5, sqrt, reciprocal, 3 mul: 10)   =  76
#   area of the quadrilateral:  2 fan triangles x 36 (c-a 3, cross 9, three dots 15, D 3,
#                               complex product 6) + b-a and a.b once (8)                      =  80
#   arctangent and doubling:    division, reduction, ~10-term series                          =  28
CLIP_FP64_FLOPS_PER_PAIR = 312


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--fields", type=int, default=128)
    p.add_argument("--layout", default="cell_major", choices=["field_major", "cell_major"])
    p.add_argument("--nside", type=int, default=256)
    p.add_argument("--dlon", type=float, default=0.25)
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the summaries of the smaller configurations in the default line")
    p.add_argument("--profile", action="store_true",
                   help="only build and run `steps` forward+transpose SpMM rounds (for an ncu capture)")
    p.add_argument("--dtype", default="float32", choices=["float32", "bfloat16"],
                   help="field type of the --profile rounds")
    p.add_argument("--pair", default="c5", choices=["c5", "identity"],
                   help="profile grids: the workload, or the 0.25-degree lon-lat grid onto itself (a diagonal "
                        "matrix, i.e. a permuted copy, to calibrate the SpMM against plain bandwidth)")
    p.add_argument("--workload", default="c5", choices=["c5", "c3", "c1", "c4", "se", "fields"],
                   help="c5: the headline (HEALPix 256 <-> 0.25 degree, 128 fields); c3: 32 jittered lon-lat "
                        "pairs of uneven resolution built as one batch and applied as one CUDA graph; c1: the "
                        "small FP64 case (2 degree -> shifted 3 degree lon-lat), build and plain FP64 apply; c4: the "
                        "differentiation case (jittered C96 <- 1 degree): adjoint apply and vertex gradients; se: "
                        "spectral-element C48 (nq 4) <-> 0.5 degree lon-lat, both builds, the oracle's beside them; "
                        "fields: the headline matrix applied to 1 .. 512 cell-major fields of FP32, BF16 and FP64")
    return p.parse_args()


def run_profile(a):
    """Build R, make the fields, run a.steps rounds of forward + transpose
    SpMM and print per-launch times and the merge-path layout statistics."""
    import torch

    from crg import Regridder, regrid_

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    hp, ll = grids_c5(a.nside, a.dlon)
    if a.pair == "identity":
        hp = ll
    R = Regridder(hp, ll, normalize=True)
    T = R.transpose()
    K, nd, ns = a.fields, R.shape[0], R.shape[1]
    gen = torch.Generator(device=dev).manual_seed(0)
    if a.layout == "cell_major":
        src = torch.randn((ns, K), generator=gen, device=dev)
        dsrc = torch.randn((nd, K), generator=gen, device=dev)
        out_f = torch.empty((nd, K), device=dev)
        out_r = torch.empty((ns, K), device=dev)
        dims = 1
    else:
        src = torch.randn((K, ns), generator=gen, device=dev)
        dsrc = torch.randn((K, nd), generator=gen, device=dev)
        out_f = torch.empty((K, nd), device=dev)
        out_r = torch.empty((K, ns), device=dev)
        dims = 2
    elem = 4
    if a.dtype == "bfloat16":
        src, dsrc = src.bfloat16(), dsrc.bfloat16()
        out_f, out_r = out_f.bfloat16(), out_r.bfloat16()
        elem = 2
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    bf, br = step_bytes(R.nnz, nd, ns, K, elem=elem)
    reps = 8  # back-to-back launches per direction keep the GPU busy past the host call overhead
    for i in range(a.steps):
        regrid_(out_f, R, src, dims=dims)
        ev[0].record()
        for _ in range(reps):
            regrid_(out_f, R, src, dims=dims)
        ev[1].record()
        for _ in range(reps):
            regrid_(out_r, T, dsrc, dims=dims)
        ev[2].record()
        ev[2].synchronize()
        tf, tr = ev[0].elapsed_time(ev[1]) / reps, ev[1].elapsed_time(ev[2]) / reps
        print(json.dumps({"round": i, "fwd_ms": tf, "rev_ms": tr, "fwd_GBs": bf / tf / 1e6, "rev_GBs": br / tr / 1e6}))
    info = {k: R.info[k] for k in ("nnz", "merge_tasks", "cut_rows", "carry_slots", "n_dst", "n_src")}
    print(json.dumps(info))


def grids_c5(nside, dlon):
    from crg import workloads

    return workloads.large(nside, dlon)


def step_bytes(nnz, nd, ns, K, elem=4, idx=4, wbytes=4):
    """Algorithmic bytes of forward + transpose."""
    fwd = nnz * (idx + wbytes) + 4 * (nd + 1) + elem * K * (ns + nd)
    rev = nnz * (idx + wbytes) + 4 * (ns + 1) + elem * K * (ns + nd)
    return fwd, rev


# ----------------------------------------------------------------- synthetic fields

def cell_centres(g):
    from crg import workloads

    return workloads.cell_centres(g)


def sh_fields(centres, K, lmax, seed, noise, device):
    from crg import workloads

    return workloads.harmonic_fields(centres, K, lmax, seed, noise, device)


# ----------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- our arm

def run_ours(a, rank, world):
    import torch

    from crg import Regridder, regrid_, regrid_batch_

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    hp, ll = grids_c5(a.nside, a.dlon)

    # --- build: warm once, then time (host grid arrays -> device CSR/CSC + apply layouts)
    R = Regridder(hp, ll, normalize=True)
    builds = []
    for i in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        torch.cuda.nvtx.range_push(f"build{i}")  # NVTX ranges select launches for ncu's launch list
        Rb = Regridder(hp, ll, normalize=True)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        builds.append(time.perf_counter() - t0)
        info = Rb.info
        del Rb
    build_s = statistics.median(builds)
    nnz, nd, ns = R.nnz, R.shape[0], R.shape[1]
    T = R.transpose()
    K = a.fields

    # --- fields: (cells, fields) cell-major (dims=1) or (fields, cells) field-major (dims=2)
    src_fm = sh_fields(cell_centres(ll), K, 64, 1, 0.1, dev)   # (K, ns): input of R
    dsrc_fm = sh_fields(cell_centres(hp), K, 64, 2, 0.1, dev)  # (K, nd): input of transpose(R)

    def layout(fm_src, fm_dsrc, cell_major):
        if cell_major:
            return (fm_src.T.contiguous(), fm_dsrc.T.contiguous(), torch.empty((nd, K), device=dev),
                    torch.empty((ns, K), device=dev), 1)
        return fm_src, fm_dsrc, torch.empty((K, nd), device=dev), torch.empty((K, ns), device=dev), 2

    cm = a.layout == "cell_major"
    src, dsrc, out_f, out_r, dims = layout(src_fm, dsrc_fm, cm)

    def step():
        regrid_(out_f, R, src, dims=dims)
        regrid_(out_r, T, dsrc, dims=dims)

    with ClockSampler(dev.index) as clk:
        # untimed warm-up: at least `warmup` steps and at least 1.5 s, so that the
        # clock sampler (100 ms period) has samples under load before timing starts
        t_w = time.perf_counter()
        n_w = 0
        while n_w < max(a.warmup, 3) or time.perf_counter() - t_w < 1.5:
            step()
            n_w += 1
            if n_w % 50 == 0:
                torch.cuda.synchronize()
        # per-direction launch times (each direction is one apply: the merge-path
        # kernel, its carry fixup and the empty-row fill, back to back on `stream`)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        kf, kr = [], []
        for _ in range(5):
            ev[0].record(stream)
            regrid_(out_f, R, src, dims=dims)
            ev[1].record(stream)
            regrid_(out_r, T, dsrc, dims=dims)
            ev[2].record(stream)
            ev[2].synchronize()
            kf.append(ev[0].elapsed_time(ev[1]))
            kr.append(ev[1].elapsed_time(ev[2]))
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("timed_steps")
        start.record(stream)
        for _ in range(a.steps):
            step()
        stop.record(stream)
        stop.synchronize()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
    ms = max_over_ranks(start.elapsed_time(stop) / a.steps, world, dev)
    bf, br = step_bytes(nnz, nd, ns, K)
    value = job_rate(world, bf + br, ms)
    # one more timed window of back-to-back launches per direction for the roofline;
    # one untimed apply first keeps the GPU busy while the host issues the timed
    # ones, so the window holds device time only (not the host's first call)
    reps = 20
    regrid_(out_f, R, src, dims=dims)
    ev[0].record(stream)
    for _ in range(reps):
        regrid_(out_f, R, src, dims=dims)
    ev[1].record(stream)
    for _ in range(reps):
        regrid_(out_r, T, dsrc, dims=dims)
    ev[2].record(stream)
    ev[2].synchronize()
    kfb, krb = ev[0].elapsed_time(ev[1]) / reps, ev[1].elapsed_time(ev[2]) / reps

    # --- accuracy against the FP64 apply (the FP64 path is bit-exact with the oracle, see tests)
    src64 = src.double()
    out64 = torch.empty(out_f.shape, dtype=torch.float64, device=dev)
    regrid_(out64, R, src64, dims=dims)
    f32 = out_f.double()
    max_abs = float((f32 - out64).abs().max() / out64.abs().max())
    ad = torch.as_tensor(R.dst_areas, device=dev)
    as_ = torch.as_tensor(R.src_areas, device=dev)
    fa = 0 if dims == 1 else 1
    wshape_d = ad[:, None] if dims == 1 else ad[None, :]
    wshape_s = as_[:, None] if dims == 1 else as_[None, :]
    tot_ref = (out64 * wshape_d).sum(dim=fa)
    tot = (f32 * wshape_d).sum(dim=fa)
    tot_src = (src64 * wshape_s).sum(dim=fa)
    cons_err = float(((tot - tot_ref).abs() / tot_ref.abs()).max())
    cons_err_src = float(((tot - tot_src).abs() / tot_src.abs()).max())
    del src64, out64

    # --- bf16 fields (FP32 accumulation) on the same layout
    sb, db = src.bfloat16(), dsrc.bfloat16()
    ob_f = torch.empty(out_f.shape, dtype=torch.bfloat16, device=dev)
    ob_r = torch.empty(out_r.shape, dtype=torch.bfloat16, device=dev)
    for _ in range(3):  # both directions: the first apply of each may time its kernel candidates
        regrid_(ob_f, R, sb, dims=dims)
        regrid_(ob_r, T, db, dims=dims)
    ev[0].record(stream)
    for _ in range(reps):
        regrid_(ob_f, R, sb, dims=dims)
        regrid_(ob_r, T, db, dims=dims)
    ev[1].record(stream)
    ev[1].synchronize()
    ms_bf16 = ev[0].elapsed_time(ev[1]) / reps
    bbf, bbr = step_bytes(nnz, nd, ns, K, elem=2)
    bf16_err = float((ob_f.double() - out_f.double()).abs().max() / out_f.double().abs().max())
    del sb, db, ob_f, ob_r

    # --- the other layout, same fields
    src2, dsrc2, of2, or2, dims2 = layout(src_fm, dsrc_fm, not cm)
    for _ in range(3):
        regrid_(of2, R, src2, dims=dims2)
        regrid_(or2, T, dsrc2, dims=dims2)
    ev[0].record(stream)
    for _ in range(reps):
        regrid_(of2, R, src2, dims=dims2)
    ev[1].record(stream)
    for _ in range(reps):
        regrid_(or2, T, dsrc2, dims=dims2)
    ev[2].record(stream)
    ev[2].synchronize()
    other = {"layout": "field_major" if cm else "cell_major",
             "ms_forward": round(ev[0].elapsed_time(ev[1]) / reps, 4),
             "ms_transpose": round(ev[1].elapsed_time(ev[2]) / reps, 4)}
    other["GB/s"] = round((bf + br) / ((other["ms_forward"] + other["ms_transpose"]) * 1e-3) / 1e9, 1)
    del src2, dsrc2, of2, or2

    # --- plain FP64, one field per launch
    s1 = src.double()[:, 0].contiguous() if dims == 1 else src.double()[0]
    r1 = dsrc.double()[:, 0].contiguous() if dims == 1 else dsrc.double()[0]
    d1 = torch.empty(nd, dtype=torch.float64, device=dev)
    o1 = torch.empty(ns, dtype=torch.float64, device=dev)
    for _ in range(3):
        regrid_(d1, R, s1)
        regrid_(o1, T, r1)
    n64 = 20
    start.record(stream)
    for _ in range(n64):
        regrid_(d1, R, s1)
        regrid_(o1, T, r1)
    stop.record(stream)
    stop.synchronize()
    ms64 = start.elapsed_time(stop) / n64
    b64f = nnz * 12 + 4 * (nd + 1) + 8 * (ns + nd) + 8 * nd
    b64r = nnz * 12 + 4 * (ns + 1) + 8 * (ns + nd) + 8 * ns
    fp64_gbs = (b64f + b64r) / (ms64 * 1e-3) / 1e9

    # --- plain FP64, all K fields in one launch per direction (cell-major; the reference's bits)
    fp64_batched = None
    if dims == 1:
        x64, dx64 = src.double(), dsrc.double()
        y64 = torch.empty((nd, K), dtype=torch.float64, device=dev)
        z64 = torch.empty((ns, K), dtype=torch.float64, device=dev)
        for _ in range(3):
            regrid_(y64, R, x64, dims=1)
            regrid_(z64, T, dx64, dims=1)
        nb = 5
        start.record(stream)
        for _ in range(nb):
            regrid_(y64, R, x64, dims=1)
            regrid_(z64, T, dx64, dims=1)
        stop.record(stream)
        stop.synchronize()
        msb = start.elapsed_time(stop) / nb
        bb = (nnz * 12 + 4 * (nd + 1) + 8 * K * (ns + nd) + 8 * nd) + (nnz * 12 + 4 * (ns + 1) + 8 * K * (ns + nd) + 8 * ns)
        # FP64 work: a product and a sum per entry and field, a division per output element
        flops = K * (2 * nnz + nd) + K * (2 * nnz + ns)
        p64 = fp64_peak()
        fp64_batched = {"ms_per_step": round(msb, 4), "GB/s": round(bb / (msb * 1e-3) / 1e9, 1),
                        "fields_per_s": round(2 * K / (msb * 1e-3), 1),
                        "speedup_vs_one_field_per_launch": round(K * ms64 / msb, 2),
                        "roofline": {"bound": "fp64", "achieved": round(flops / (msb * 1e-3) / 1e12, 4),
                                     "peak": round(p64, 4), "unit": "TFLOP/s",
                                     "frac": round(flops / (msb * 1e-3) / 1e12 / p64, 4),
                                     "flops_per_step": flops,
                                     "note": "unfused product and sum per entry (the reference's rounding), "
                                             "one division per output element"}}
        del x64, dx64, y64, z64

    # --- e2e through the public API with pinned host buffers (copies inside the timed region)
    hs = src.cpu().pin_memory()
    hd = dsrc.cpu().pin_memory()
    ho_f = torch.empty(tuple(out_f.shape), dtype=torch.float32).pin_memory()
    ho_r = torch.empty(tuple(out_r.shape), dtype=torch.float32).pin_memory()

    # the step's two applies are independent (different inputs): one public call
    # runs them concurrently, so their copies share both directions of the link
    def step_host():
        regrid_batch_([(ho_f, R, hs, dims), (ho_r, T, hd, dims)])

    def step_host_sequential():
        regrid_(ho_f, R, hs, dims=dims)
        regrid_(ho_r, T, hd, dims=dims)

    def timed(step):
        """Median over 5 windows of ne steps (3 warm-up steps first), and the
        windows' range."""
        for _ in range(3):
            step()
        torch.cuda.synchronize()
        ne = max(3, min(a.steps, 6))
        ws = []
        for _ in range(5):
            t0 = time.perf_counter()
            for _ in range(ne):
                step()
            torch.cuda.synchronize()
            ws.append((time.perf_counter() - t0) * 1e3 / ne)
        return statistics.median(ws), (min(ws), max(ws))

    e2e_seq_ms, _ = timed(step_host_sequential)
    e2e_ms, e2e_range = timed(step_host)
    h2d = 4 * K * (ns + nd)
    d2h = 4 * K * (nd + ns)
    assert torch.equal(ho_f, out_f.cpu()), "host-buffer apply differs from the device apply"
    assert torch.equal(ho_r, out_r.cpu()), "host-buffer transpose apply differs from the device apply"
    # link ceiling: plain pinned copies of the same bytes
    gb = torch.empty(hs.shape, device=dev)
    ev[0].record(stream)
    gb.copy_(hs, non_blocking=True)
    ev[1].record(stream)
    hs.copy_(gb, non_blocking=True)
    ev[2].record(stream)
    ev[2].synchronize()
    link = {"h2d_GBs": round(hs.numel() * 4 / ev[0].elapsed_time(ev[1]) / 1e6, 1),
            "d2h_GBs": round(hs.numel() * 4 / ev[1].elapsed_time(ev[2]) / 1e6, 1)}
    # both directions at once (the step's copies overlap in and out): the
    # ceiling the e2e number is compared with
    gb2 = torch.empty(hs.shape, device=dev)
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    best = None
    for _ in range(3):
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        s_in.wait_event(t0)
        s_out.wait_event(t0)
        with torch.cuda.stream(s_in):
            gb.copy_(hs, non_blocking=True)
        with torch.cuda.stream(s_out):
            ho_r.copy_(gb2, non_blocking=True)  # ho_r was checked above; its contents are not used again
        stream.wait_stream(s_in)
        stream.wait_stream(s_out)
        t1.record(stream)
        t1.synchronize()
        best = t0.elapsed_time(t1) if best is None else min(best, t0.elapsed_time(t1))
    link["duplex_GBs"] = round(2 * hs.numel() * 4 / best / 1e6, 1)
    del gb2

    peak, peak_source = hbm_peak()
    launch_ms = (kfb + krb) / 2
    achieved = ((bf + br) / 2) / (launch_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": round(ms, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32",
        "data": "synthetic: degree-64 spherical harmonics + N(0,0.1) noise",
        "config": {"workload": WORKLOAD, "n_dst": nd, "n_src": ns, "nnz": nnz, "fields": K, "layout": a.layout,
                   "l2": "inputs 0.9 GB per direction > 129 MB L2, no flush", "parallelism": f"replicas x{world}",
                   "weights": "fp32, FP64-built", "accumulate": "fp32", "value": VALUE_DEF},
        "fields_per_s": round(world * 2 * K / (ms * 1e-3), 1),
        "build": {"ms": round(build_s * 1e3, 3), "pairs_per_s": round(nnz / build_s, 1),
                  "candidates": info["n_candidates"], "clipped": info["n_clipped"],
                  "search_ms": round(info["t_search_ms"], 3),
                  "clip_ms": round(info["t_clip_ms"], 3), "assemble_ms": round(info["t_assemble_ms"], 3),
                  "roofline": build_roofline(info)},
        "fp64_one_field_per_launch": {"ms_per_field_both_directions": round(ms64, 4), "GB/s": round(fp64_gbs, 2),
                                      "fields_per_s": round(2 / (ms64 * 1e-3), 1)},
        "fp64_batched": fp64_batched,
        "bf16": {"ms_per_step": round(ms_bf16, 4), "GB/s": round((bbf + bbr) / (ms_bf16 * 1e-3) / 1e9, 1),
                 "fields_per_s": round(2 * K / (ms_bf16 * 1e-3), 1), "max_abs_err_vs_fp32_rel_to_max": bf16_err},
        "other_layout": other,
        "accuracy_vs_fp64": {"max_abs_err_rel_to_max": max_abs, "mean_conservation_rel_err": cons_err,
                             "mean_conservation_rel_err_vs_src_total": cons_err_src},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": profiled_traffic(a),
                     "kernel": "k_cm_nnz (launch_ms: each direction's launches, incl. k_cm_fixup for cut rows)"
                     if a.layout == "cell_major" else "k_fm_rows",
                     "launch_ms": {"forward": round(kfb, 4), "transpose": round(krb, 4)},
                     "algorithmic_bytes_per_launch": {"forward": bf, "transpose": br},
                     "peak_source": peak_source},
        "e2e": {"value": round(world * (bf + br) / (e2e_ms * 1e-3) / 1e9, 2), "unit": "GB/s",
                "ms_per_step": round(e2e_ms, 3), "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step_range": [round(e2e_range[0], 3), round(e2e_range[1], 3)],
                "timing": "median of 5 windows of 6 steps after 3 warm-up steps (wall clock, synchronised)",
                "call": "regrid_batch_ (crg_apply_batch) of the step's two applies, pinned host fields",
                "sequential": {"ms_per_step": round(e2e_seq_ms, 3),
                               "GB/s": round(world * (bf + br) / (e2e_seq_ms * 1e-3) / 1e9, 2),
                               "call": "regrid_ then regrid_"},
                "link_probe": link,
                "link_frac": round((h2d + d2h) / (e2e_ms * 1e-3) / 1e9 / link["duplex_GBs"], 4)},
        "gpu_launches": a.steps * launches_per_step(R.info, K, a.layout),
        "clocks": clk.summary(),
    }
    del hs, hd, ho_f, ho_r, gb, src, dsrc, out_f, out_r, src_fm, dsrc_fm
    if rank == 0 and not a.no_configs:
        # the smaller configurations, summarised (each is also `--workload c1|c3|c4`)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        line["configs"] = {"small_fp64": run_c1(a), "batches": run_c3(a), "derivatives": run_c4(a)}
    if rank == 0 and not a.no_cpu:
        line["cpu_baseline"] = cpu_baseline(hp, ll, K, sample_fields=16)
    return line


def hbm_peak():
    """The HBM roofline denominator: the machine's measured copy bandwidth, or the
    stated fallback when the measurement file is absent."""
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        peaks = json.loads(f.read_text())
        if peaks.get("hbm_gbs"):
            return float(peaks["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
    return 6800.0, "fallback 6.8 TB/s (of fallback: MEASURED_PEAKS.json absent)"


def fp64_peak():
    """FP64 TFLOP/s of this GPU from our own FMA-loop kernel (k_fp64_fma in
    crg_peaks.cu, best of 5 launches of 1e10 FLOPs)."""
    import ctypes

    from crg import _build

    lib = ctypes.CDLL(str(_build.PEAKS_LIB_PATH))
    lib.crg_peak_fp64_tflops.restype = ctypes.c_int
    lib.crg_peak_fp64_tflops.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    t, ms = ctypes.c_double(), ctypes.c_double()
    rc = lib.crg_peak_fp64_tflops(5, ctypes.byref(t), ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError(f"crg_peak_fp64_tflops failed with CUDA error {rc}")
    return t.value


def build_roofline(info):
    """The clip kernel against the FP64 pipe: CLIP_FP64_FLOPS_PER_PAIR x the
    pairs it clips, over its CUDA-event time inside the build (the span from
    the end of the search to the end of k_clip, which also holds three small
    counter memsets)."""
    peak = fp64_peak()
    pairs = int(info["n_clipped"])
    ms = float(info["t_clip_ms"])
    achieved = CLIP_FP64_FLOPS_PER_PAIR * pairs / (ms * 1e-3) / 1e12
    return {"bound": "fp64", "achieved": round(achieved, 4), "peak": round(peak, 4), "unit": "TFLOP/s",
            "frac": round(achieved / peak, 4), "kernel": "k_clip", "flops_per_pair": CLIP_FP64_FLOPS_PER_PAIR,
            "pairs": pairs, "launch_ms": round(ms, 4),
            "peak_source": "k_fp64_fma (crg_peaks.cu), measured in this run (of measured)"}


def max_over_ranks(ms, world, device):
    """The slowest replica's time per step (every rank gets it)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, bytes_per_step, ms):
    """Whole-job GB/s: every replica moves bytes_per_step per step, the job
    takes the slowest replica's time."""
    return world * bytes_per_step / (ms * 1e-3) / 1e9


def launches_per_step(info, K, layout):
    """Kernels one forward + transpose step launches: per 128-field pass the
    merge-path kernel and, when the direction has rows cut between tasks, their
    fixup; one zero fill per direction with empty rows (field-major: one row
    kernel per direction)."""
    if layout != "cell_major":
        return 2
    passes = (K + 127) // 128
    n = 0
    for d in range(2):
        n += passes * (1 + (info["cut_rows"][d] > 0)) + (info["empty_rows"][d] > 0)
    return n


def profiled_traffic(a):
    """DRAM bytes (read + write) of one k_cm_nnz launch on this workload, from
    the ncu summary kept beside the code; None when there is none for it."""
    f = ROOT / "profiles" / "k_cm_nnz_healpix256_lonlat025_k128.md"
    if a.layout != "cell_major" or a.fields != 128 or a.nside != 256 or a.dlon != 0.25 or not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            return int(line.split(":")[1].strip())
    return None


# ----------------------------------------------------------------- batched workload

def run_c3(a):
    """Build the 32 pairs one at a time and as one batch; apply every pair's
    fields one call at a time and as one captured graph (forward direction,
    cell-major FP32 fields, inputs resident on the device)."""
    import torch

    from crg import ApplyPlan, Regridder, build_batch, regrid_

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    from crg import workloads

    pairs, ks = workloads.batch_pairs()
    build_batch(pairs[:2])  # warm the library and the allocator
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    single = [Regridder(d, s, normalize=True) for d, s in pairs]
    torch.cuda.synchronize()
    t_single = time.perf_counter() - t0
    del single
    t0 = time.perf_counter()
    Rs = build_batch(pairs, normalize=True, nthreads=8)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    nnz = sum(R.nnz for R in Rs)
    gen = torch.Generator(device=dev).manual_seed(5)
    items, nbytes = [], 0
    for R, K in zip(Rs, ks):
        nd, ns = R.shape
        shp_in, shp_out = ((ns,), (nd,)) if K == 1 else ((ns, K), (nd, K))
        x = torch.randn(shp_in, generator=gen, device=dev)
        y = torch.empty(shp_out, device=dev)
        items.append((y, R, x, 1))
        nbytes += step_bytes(R.nnz, nd, ns, K)[0]
    plan = ApplyPlan(items)
    # for comparison: every item as its own graph branch, and every item in the
    # persistent launch
    forms = {}
    for form, env in (("branches", "0"), ("all", "all")):
        os.environ["CRG_PLAN_BATCH"] = env
        try:
            forms[form] = ApplyPlan(items)
        finally:
            del os.environ["CRG_PLAN_BATCH"]
    plan_branches, plan_all = forms["branches"], forms["all"]

    def loop():
        for y, R, x, dims in items:
            regrid_(y, R, x, dims=dims)

    stream = torch.cuda.current_stream(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    for _ in range(max(a.warmup, 3)):
        loop()
        plan.launch()
        plan_branches.launch()
        plan_all.launch()
    reps = max(5, min(a.steps, 50))
    torch.cuda.synchronize()
    ev[0].record(stream)
    for _ in range(reps):
        loop()
    ev[1].record(stream)
    for _ in range(reps):
        plan.launch()
    ev[2].record(stream)
    ev[2].synchronize()
    ms_loop = ev[0].elapsed_time(ev[1]) / reps
    ms_plan = ev[1].elapsed_time(ev[2]) / reps
    ev[0].record(stream)
    for _ in range(reps):
        plan_branches.launch()
    ev[1].record(stream)
    ev[1].synchronize()
    ms_branches = ev[0].elapsed_time(ev[1]) / reps
    ev[0].record(stream)
    for _ in range(reps):
        plan_all.launch()
    ev[1].record(stream)
    ev[1].synchronize()
    ms_all = ev[0].elapsed_time(ev[1]) / reps
    # one replay of each plan inside an NVTX range (selects their launches for ncu's launch list)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("c3_plan")
    plan.launch()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    torch.cuda.nvtx.range_push("c3_branches")
    plan_branches.launch()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    cells = [(R.shape[0], R.shape[1]) for R in Rs]
    return {
        "metric": "batched build pairs/s (summed) and batched apply GB/s",
        "workload": "32 jittered global lon-lat pairs, resolution exp(U[ln 0.4, ln 4]) deg per side, "
                    "K = round(exp(U[0, ln 512])) fp32 fields, forward applies",
        "pairs": 32, "nnz_total": nnz, "fields_total": int(sum(ks)),
        "cells_min_max": [int(min(min(c) for c in cells)), int(max(max(c) for c in cells))],
        "build": {"single_ms": round(t_single * 1e3, 2), "batch_ms": round(t_batch * 1e3, 2),
                  "pairs_per_s_batch": round(nnz / t_batch, 1), "pairs_per_s_single": round(nnz / t_single, 1)},
        "apply": {"loop_ms": round(ms_loop, 4), "graph_ms": round(ms_plan, 4),
                  "GB/s_graph": round(nbytes / (ms_plan * 1e-3) / 1e9, 1),
                  "GB/s_loop": round(nbytes / (ms_loop * 1e-3) / 1e9, 1), "bytes_per_batch": nbytes,
                  "graph_kernels": plan.info["kernels"], "graph_batched_items": plan.info["batched_items"],
                  "graph": "one CUDA graph: the small multi-pass pairs in one persistent launch, every other "
                           "pair its own tuned apply on a branch",
                  "branches_ms": round(ms_branches, 4), "branches_kernels": plan_branches.info["kernels"],
                  "GB/s_branches": round(nbytes / (ms_branches * 1e-3) / 1e9, 1),
                  "all_persistent_ms": round(ms_all, 4), "all_persistent_kernels": plan_all.info["kernels"],
                  "GB/s_all_persistent": round(nbytes / (ms_all * 1e-3) / 1e9, 1)},
    }


def run_fields(a):
    """The headline matrix (HEALPix 256 <-> 0.25 degree) applied forward and
    transposed to K cell-major fields, K = 1 .. 512, FP32, BF16 and FP64: CUDA-
    event time per step (both directions, inputs resident, larger than L2 from
    K = 64 FP32) and the algorithmic bytes per second."""
    import torch

    from crg import Regridder, regrid_

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    hp, ll = grids_c5(a.nside, a.dlon)
    R = Regridder(hp, ll, normalize=True)
    T = R.transpose()
    nnz, nd, ns = R.nnz, R.shape[0], R.shape[1]
    peak, peak_source = hbm_peak()
    gen = torch.Generator(device=dev).manual_seed(9)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    out = []
    for dt, elem, wb in ((torch.float32, 4, 4), (torch.bfloat16, 2, 4), (torch.float64, 8, 8)):
        for K in (1, 2, 4, 8, 16, 32, 64, 128, 256, 512):
            if dt == torch.float64 and K > 128:
                continue
            shp = (lambda n: (n,)) if K == 1 else (lambda n: (n, K))
            x = torch.randn(shp(ns), generator=gen, device=dev).to(dt)
            z = torch.randn(shp(nd), generator=gen, device=dev).to(dt)
            y, w = torch.empty(shp(nd), dtype=dt, device=dev), torch.empty(shp(ns), dtype=dt, device=dev)
            for _ in range(3):
                regrid_(y, R, x)
                regrid_(w, T, z)
            reps = 10
            ev[0].record()
            for _ in range(reps):
                regrid_(y, R, x)
                regrid_(w, T, z)
            ev[1].record()
            ev[1].synchronize()
            ms = ev[0].elapsed_time(ev[1]) / reps
            bf, br = step_bytes(nnz, nd, ns, K, elem=elem, wbytes=wb)
            gbs = (bf + br) / (ms * 1e-3) / 1e9
            out.append({"dtype": str(dt).replace("torch.", ""), "fields": K, "ms_per_step": round(ms, 4),
                        "GB/s": round(gbs, 1), "frac_of_hbm": round(gbs / peak, 3)})
            del x, z, y, w
    return {"metric": "apply GB/s over field counts (forward + transpose, cell-major)",
            "workload": WORKLOAD.split(",")[0] + ", K fields", "peak_GBs": peak, "peak_source": peak_source,
            "bytes": "8 B per nonzero (FP32 weight and column; FP64: 12 B) + row pointers + K x elem x (rows + "
                     "columns) per direction", "results": out}


# ----------------------------------------------------------------- small FP64 workload

def run_c1(a):
    """2-degree lon-lat source, 3-degree destination shifted by (+0.7, +0.4)
    degrees with latitude edges clamped to the poles; normalize = true; one
    FP64 field U[0, 1).  Build pairs/s and candidates/s (median of 20 builds),
    FP64 apply GB/s (bytes 12 nnz + 4 (rows + 1) + 8 (cols + rows) + 8 rows)."""
    import torch

    from crg import Regridder, grids, regrid_

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    src = grids.lonlat_regular(2.0, 2.0)
    dst = grids.lonlat_grid(0.7 + 3 * np.arange(121), np.clip(-89.6 + 3 * np.arange(61), -90, 90))
    Regridder(dst, src, normalize=True)
    times = []
    for _ in range(20):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        R = Regridder(dst, src, normalize=True)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    tb = statistics.median(times)
    nd, ns = R.shape
    s = torch.rand(ns, dtype=torch.float64, device=dev, generator=torch.Generator(device=dev).manual_seed(1))
    d = torch.empty(nd, dtype=torch.float64, device=dev)
    for _ in range(max(a.warmup, 3)):
        regrid_(d, R, s)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 200
    e0.record(stream)
    for _ in range(reps):
        regrid_(d, R, s)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nbytes = 12 * R.nnz + 4 * (nd + 1) + 8 * (ns + nd) + 8 * nd
    return {"metric": "small FP64 build pairs/s and apply GB/s", "workload": "lonlat 2deg -> lonlat 3deg shifted, fp64",
            "n_dst": nd, "n_src": ns, "nnz": R.nnz, "candidates": R.info["n_candidates"],
            "build": {"ms_median": round(tb * 1e3, 3), "pairs_per_s": round(R.nnz / tb, 1),
                      "candidates_per_s": round(R.info["n_candidates"] / tb, 1)},
            "apply_fp64": {"ms": round(ms, 4), "GB/s": round(nbytes / (ms * 1e-3) / 1e9, 2),
                           "note": "one launch of ~16 K rows: launch-latency bound"}}


def run_c4(a):
    """Differentiation: jittered C96 cubed sphere (vertices moved by U(-0.15,
    0.15) cell widths, seed 11) <- 1-degree lon-lat, FP64, one field.  The
    adjoint apply A^T (g ./ a) in GB/s (bytes 12 nnz + 4 (rows + 1) +
    8 (cols + rows) + 8 rows, CUDA events over 200 launches), and the median
    wall time of the destination-vertex area gradient (crg_area_grad), the
    source-vertex one (crg_area_grad of the swapped regridder, built once)
    and the whole pullback of L = sum w d^2 (host arrays in and out)."""
    import torch

    from crg import Regridder, area_grad, grids, regrid_, regrid_adjoint_, regrid_pullback, src_area_grad

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    dst, src = grids.cubed_sphere(96, jitter=0.15, seed=11), grids.lonlat_regular(1.0, 1.0)
    R = Regridder(dst, src, normalize=True)
    times = []
    for _ in range(5):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        R = Regridder(dst, src, normalize=True)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    tb = statistics.median(times)
    nd, ns = R.shape
    rng = np.random.default_rng(2024)
    s, w = rng.standard_normal(ns), rng.standard_normal(nd)
    d = np.zeros(nd)
    regrid_(d, R, s)
    g = 2.0 * w * d
    gd = torch.from_numpy(g).to(dev)
    sb = torch.empty(ns, dtype=torch.float64, device=dev)
    for _ in range(max(a.warmup, 3)):
        regrid_adjoint_(sb, R, gd)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 200
    e0.record(stream)
    for _ in range(reps):
        regrid_adjoint_(sb, R, gd)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nbytes = 12 * R.nnz + 4 * (ns + 1) + 8 * (nd + ns) + 8 * nd
    a_un = R.dst_areas * (R.info["normalizer"] if R.info["normalized"] else 1.0)
    u, c = g / a_un, -g * d / a_un
    Rs = Regridder(src, dst)

    def median_s(fn, n=5):
        fn()
        out = []
        for _ in range(n):
            t0 = time.perf_counter()
            fn()
            out.append(time.perf_counter() - t0)
        return statistics.median(out)

    t_v = median_s(lambda: area_grad(R, dst, src, u, s, c))
    t_w = median_s(lambda: src_area_grad(dst, src, u, s, swapped=Rs))
    t_p = median_s(lambda: regrid_pullback(R, dst, src, s, g, wrt_src=True, swapped=Rs), n=3)
    return {"metric": "differentiation: adjoint apply GB/s and vertex-gradient times",
            "workload": "jittered C96 cubed sphere <- lonlat 1deg, fp64, 1 field",
            "n_dst": nd, "n_src": ns, "nnz": R.nnz,
            "build": {"ms_median": round(tb * 1e3, 3), "pairs_per_s": round(R.nnz / tb, 1)},
            "adjoint_fp64": {"ms": round(ms, 4), "GB/s": round(nbytes / (ms * 1e-3) / 1e9, 2)},
            "area_grad_dst": {"ms_median": round(t_v * 1e3, 3), "nonzeros_per_s": round(R.nnz / t_v, 1),
                              "note": "host arrays in and out; 4 destination vertices per nonzero, one dual pass each"},
            "area_grad_src": {"ms_median": round(t_w * 1e3, 3), "nonzeros_per_s": round(Rs.nnz / t_w, 1)},
            "pullback_all": {"ms_median": round(t_p * 1e3, 3),
                             "note": "apply + adjoint + both vertex gradients (swapped regridder reused)"}}


def run_se(a):
    """Spectral-element C48 space with 4 x 4 GLL nodes per element (ClimaCore
    CubedSphereSpace(h_elem = 48, n_quad_points = 4)) and the 0.5-degree
    lon-lat grid: SE -> FV principled and FV -> SE L2-projection builds
    (median of 5 each, pairs = nonzeros), the FP64 apply of one field each way,
    and the oracle's builds (all host threads) of the same pair."""
    import torch

    from crg import Regridder, SpectralElementSpace, grids, regrid_

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    space, fv = SpectralElementSpace.cubed_sphere(48, 4), grids.lonlat_regular(0.5, 0.5)
    out = {"metric": "SE <-> FV build pairs/s", "workload": "cubed sphere C48, nq 4 (36,864 nodes) <-> lonlat 0.5deg",
           "n_nodes": space.nnodes, "n_fv": fv.ncells}
    for name, make in (("se_to_fv", lambda: Regridder(fv, space)), ("fv_to_se", lambda: Regridder(space, fv))):
        make()
        times = []
        for i in range(5):
            torch.cuda.synchronize()
            torch.cuda.nvtx.range_push(f"{name}{i}")  # NVTX ranges select launches for ncu's launch list
            t0 = time.perf_counter()
            R = make()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            torch.cuda.nvtx.range_pop()
        tb = statistics.median(times)
        nd, ns = R.shape
        s = torch.rand(ns, dtype=torch.float64, device=dev, generator=torch.Generator(device=dev).manual_seed(1))
        d = torch.empty(nd, dtype=torch.float64, device=dev)
        for _ in range(max(a.warmup, 3)):
            regrid_(d, R, s)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream = torch.cuda.current_stream(dev)
        e0.record(stream)
        for _ in range(50):
            regrid_(d, R, s)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / 50
        out[name] = {"build_ms_median": round(tb * 1e3, 3), "nnz": R.nnz, "candidates": R.info["n_candidates"],
                     "pairs_per_s": round(R.nnz / tb, 1), "overlap_integrals_ms": round(R.info["t_clip_ms"], 3),
                     "apply_fp64_ms": round(ms, 4)}
    if not a.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle

        for name, se_dst in (("se_to_fv", False), ("fv_to_se", True)):
            t0 = time.perf_counter()
            O = oracle.OracleSERegridder(fv, space.elements, 4, se_dst)
            out[name]["oracle_build_s"] = round(time.perf_counter() - t0, 3)
            out[name]["oracle_threads"] = oracle.load().og_num_threads()
            out[name]["same_nnz_as_oracle"] = O.nnz == out[name]["nnz"]
    return out


# ----------------------------------------------------------------- CPU legs (oracle)

def _oracle_fields(O, K, seed=3):
    rng = np.random.default_rng(seed)
    S = rng.standard_normal((K, O.ns)).astype(np.float32)
    D = rng.standard_normal((K, O.nd)).astype(np.float32)
    return S, D, np.empty((K, O.nd), np.float32), np.empty((K, O.ns), np.float32)


def cpu_baseline(hp, ll, K, sample_fields):
    """The oracle's apply (the reference's regrid!: one CSC mul! per Float32
    field with the Float64 matrix, then ./ areas; fields over all host threads)
    on a bounded sample of the workload, in the headline's unit: the
    algorithmic FP32 bytes of a `sample_fields`-field step over its time.  The
    oracle's build of the same regridder is timed beside it."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    t0 = time.perf_counter()
    O = oracle.OracleRegridder(hp, ll, normalize=True)
    tb = time.perf_counter() - t0
    S, D, Y, Z = _oracle_fields(O, sample_fields)
    O.apply_f32(S[:1], out=Y[:1])
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        O.apply_f32(S, out=Y)
        O.apply_f32(D, transpose=True, out=Z)
    t = (time.perf_counter() - t0) / reps
    bf, br = step_bytes(O.nnz, O.nd, O.ns, sample_fields)
    cores = oracle.load().og_num_threads()
    # the reference's apply is one single-threaded mul! per field: one thread, one field
    t0 = time.perf_counter()
    O.apply_f32(S[:1], nthreads=1, out=Y[:1])
    O.apply_f32(D[:1], transpose=True, nthreads=1, out=Z[:1])
    t1 = time.perf_counter() - t0
    b1f, b1r = step_bytes(O.nnz, O.nd, O.ns, 1)
    return {"value": round((bf + br) / t / 1e9, 3), "unit": "GB/s", "cores": cores, "kind": "port",
            "sample": f"{sample_fields} of {K} fp32 fields, forward + transpose (the reference's Float32 regrid! "
                      "with its Float64 matrix), bytes as in the headline",
            "fields_per_s": round(2 * sample_fields / t, 1),
            "build": {"s": round(tb, 3), "pairs_per_s": round(O.nnz / tb, 1), "threads": cores},
            "single_thread": {"value": round((b1f + b1r) / t1 / 1e9, 3), "unit": "GB/s",
                              "sample": "1 field, forward + transpose, 1 thread"}}


def run_reference(a):
    """The reference arm: the CPU restatement of regrid! with R and
    transpose(R) on the whole step (all `a.fields` Float32 fields both ways),
    on all host threads; value = the headline's algorithmic bytes of that step
    over its time, so that it divides like for like with our arm."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    hp, ll = grids_c5(a.nside, a.dlon)
    t0 = time.perf_counter()
    O = oracle.OracleRegridder(hp, ll, normalize=True)
    tb = time.perf_counter() - t0
    K = a.fields
    S, D, Y, Z = _oracle_fields(O, K)
    for _ in range(a.warmup):
        O.apply_f32(S, out=Y)
        O.apply_f32(D, transpose=True, out=Z)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        O.apply_f32(S, out=Y)
        O.apply_f32(D, transpose=True, out=Z)
    ms = (time.perf_counter() - t0) * 1e3 / a.steps
    bf, br = step_bytes(O.nnz, O.nd, O.ns, K)
    value = (bf + br) / (ms * 1e-3) / 1e9
    cores = oracle.load().og_num_threads()
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": 0,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic: N(0,1) fields",
        "config": {"workload": WORKLOAD, "n_dst": O.nd, "n_src": O.ns, "nnz": O.nnz, "fields": K,
                   "value": VALUE_DEF, "accumulate": "fp64 products, fp32 stores (Julia mul! on Float32 arrays)"},
        "fields_per_s": round(2 * K / (ms * 1e-3), 1),
        "build": {"s": round(tb, 3), "pairs_per_s": round(O.nnz / tb, 1), "threads": cores},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": f"all {K} fp32 fields per step, forward + transpose (C restatement of the "
                                   "reference's regrid!; Julia is not installed)"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    a = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if a.profile:
        run_profile(a)
        return
    if a.workload in ("c3", "c1", "c4", "se", "fields"):
        if rank == 0:
            print(json.dumps({"c3": run_c3, "c1": run_c1, "c4": run_c4, "se": run_se,
                              "fields": run_fields}[a.workload](a)))
        return
    if a.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(a)))
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    line = run_ours(a, rank, world)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()

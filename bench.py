#!/usr/bin/env python
"""Benchmark of the GB300 domain-wall Wilson hopping term (GridBench's Dhop).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--quick]

Headline workload: FP32 Dhop on a 16^4 x Ls=16 periodic lattice with seeded random SU(3)
links and a Gaussian fermion.  One step = one application of the hopping term to the whole
lattice (1320 flop per 5D site, GridBench's own count).  Two in/out pairs alternate, so the
working set (476 MB) is well above the 129 MB L2 between consecutive steps.

The JSON line carries: value (device-timed GFLOP/s, inputs resident in HBM), the HBM
roofline of the kernel (algorithmic bytes 2*S + 8*G/(Ls*k) per 5D site), e2e (the same
metric through the public API with the step's input copied from pinned host memory and the
result copied back every step; steps rotate over three library streams so one step's
write-back overlaps the next steps' input copies), the CPU baseline (the oracle port timed on
the host cores), SM clocks sampled during the timed region, the number of kernels launched,
and secondary workloads (FP64, DhopDag, FP16 storage, even-odd, the Mobius operator, halo
packing, 12-RHS, batched persistent, and CG to a 1e-10 true residual at 32^4 x Ls=16: plain vs
mixed on M^dag M and through the even-odd Schur complement).

--impl reference times the reference's algorithm on the host CPU (the oracle port of
dslash_simple.h, all host threads) on the same workload; each step is a bounded sample of
the lattice.  Multi-GPU (torchrun, N>1) runs independent replicas (the path does not shard).
"""
from __future__ import annotations

import argparse
import datetime as _dt
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOP_PER_SITE = 1320
SPINOR_BYTES = {0: 192, 1: 96, 2: 52}  # per 5D site: F64, F32, F16 (+4 B norm)
LINK_BYTES = {0: 144, 1: 72, 2: 24, 3: 24}  # per link: F64, F32, 12-real F16/BF16
METRIC = "Dhop GFLOP/s & % HBM roofline; mixed vs plain CG time-to-1e-10 on 1 GB300"
DIMS = (16, 16, 16, 16)
LS = 16
# The workload both arms name in `config` (identical dicts: the same lattice, precision and
# working set; how each arm launches it is reported outside `config`).
CONFIG = {"workload": "FP32 domain-wall Wilson Dhop, 16^4 x Ls=16, periodic", "lattice": list(DIMS), "Ls": LS,
          "l2": "inputs larger than L2: two alternating in/out pairs, 476 MB vs 129 MB L2"}
WHY_PORT = ("the oracle port stands in for the reference's dslash_simple.h (bit-identical to it on the same inputs, "
            "checked where the reference tree exists); the reference tree is not present on the GPU host, and the "
            "reference's AVX-512/AVX2 hand kernels are x86 intrinsics that do not build on its Arm cores")


def algo_bytes(sprec: int, gprec: int, Ls: int, k: int = 1) -> float:
    """Algorithmic bytes per 5D site per right-hand side: read + write one spinor, links
    amortised over the Ls*k slices that share them (neighbour table excluded)."""
    return 2 * SPINOR_BYTES[sprec] + 8 * LINK_BYTES[gprec] / (Ls * k)


# ------------------------------------------------------------------ distributed plumbing
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            vis = os.environ.get("CUDA_VISIBLE_DEVICES")
            if vis and "," in vis:
                ids = vis.split(",")
                os.environ["CUDA_VISIBLE_DEVICES"] = ids[self.local % len(ids)]
            elif not vis:
                os.environ["CUDA_VISIBLE_DEVICES"] = str(self.local)
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ------------------------------------------------------------------ clocks during the timed region
class Clocks:
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def start(self):
        if shutil.which("nvidia-smi") is None:
            return
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0] or "0"
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(["nvidia-smi", "-i", vis, "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits", "-lms", "100"],
                                     stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        time.sleep(1.0)  # let the sampler start before the timed region

    def mark(self, which: str):
        setattr(self, which, _dt.datetime.now())

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 10:
                continue
            try:
                ts = _dt.datetime.strptime(p[0], "%Y/%m/%d %H:%M:%S.%f")
                rows.append((ts, float(p[2]), float(p[3]), p[6:10]))
            except ValueError:
                continue
        os.unlink(self.path)
        inside = [r for r in rows if self.t0 and self.t1 and self.t0 <= r[0] <= self.t1] or rows
        if not inside:
            return None
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for r in inside for i, v in enumerate(r[3]) if v.lower().startswith("active")})
        sm = sorted(r[1] for r in inside)
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[2] for r in inside), "reasons": reasons,
                "samples": len(inside)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(key: str):
    """DRAM bytes per launch from a committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(key)
    except (OSError, ValueError):
        return None


# ------------------------------------------------------------------ our arm
def cpu_baseline(dims, Ls, budget_s=10.0) -> dict:
    """The oracle port (scalar C restatement of dslash_simple.h, OpenMP over all host
    threads) on the full FP32 lattice, repeated for about budget_s seconds."""
    import oracle
    U = oracle.generate_gauge(dims).astype(np.float32)
    phi = oracle.generate_fermion(dims, Ls).astype(np.float32)
    nbr, prm, nsite = oracle.generate_table(dims, Ls)
    out = np.zeros_like(phi)
    oracle.dslash_sites(U, phi, out, nbr, 0, nsite, Ls)  # warm
    t = time.perf_counter()
    oracle.dslash_sites(U, phi, out, nbr, 0, nsite, Ls)
    one = time.perf_counter() - t
    reps = max(1, min(1000, int(budget_s / max(one, 1e-6))))
    t = time.perf_counter()
    for _ in range(reps):
        oracle.dslash_sites(U, phi, out, nbr, 0, nsite, Ls)
    dt = time.perf_counter() - t
    # the same port on one thread, for about a third of the budget
    oracle.set_threads(1)
    try:
        t = time.perf_counter()
        oracle.dslash_sites(U, phi, out, nbr, 0, nsite, Ls)
        one1 = time.perf_counter() - t
        reps1 = max(1, min(200, int(budget_s / 3 / max(one1, 1e-6))))
        t = time.perf_counter()
        for _ in range(reps1):
            oracle.dslash_sites(U, phi, out, nbr, 0, nsite, Ls)
        dt1 = time.perf_counter() - t
    finally:
        oracle.set_threads(oracle.threads())
    return {"value": round(FLOP_PER_SITE * nsite * Ls * reps / dt / 1e9, 3), "unit": "GFLOP/s",
            "cores": oracle.threads(), "kind": "port",
            "sample": f"{reps} full FP32 Dhop passes over {'x'.join(map(str, dims))} x Ls={Ls} "
                      f"({dt:.1f} s, oracle port of dslash_simple.h with OpenMP)",
            "single_thread": {"value": round(FLOP_PER_SITE * nsite * Ls * reps1 / dt1 / 1e9, 3), "cores": 1,
                              "sample": f"{reps1} passes ({dt1:.1f} s)"},
            "why_port": WHY_PORT}


def time_dhop(gb, g, pairs, steps, warmup, dag=0):
    """Device time (ms) of `steps` hopping applications alternating over (out, in) pairs."""
    for i in range(warmup):
        y, x = pairs[i % len(pairs)]
        gb.dhop(g, y, x, dag)
    gb.synchronize()
    t = gb.Timer()
    n0 = gb.launch_count()
    t.start()
    for i in range(steps):
        y, x = pairs[i % len(pairs)]
        gb.dhop(g, y, x, dag)
    ms = t.stop()
    return ms, gb.launch_count() - n0


def rel_to(gb, lat, a, b) -> float:
    """|a - b| / |b| on the device in FP64 (every right-hand side of multi-RHS fields)."""
    d = gb.Field(lat, gb.F64, a.nrhs)
    d.copy_from(a)
    bb = gb.Field(lat, gb.F64, b.nrhs)
    bb.copy_from(b)
    d.axpby(-1.0, bb, 1.0)
    return float(np.sqrt(d.norm2() / bb.norm2()))


def halo_rel_err(x32, x64) -> float:
    """Relative error of the eight FP32 halo faces of x32 against the same faces packed from
    an FP64 field holding x32's values, over all faces (both packed to host memory and
    decoded from the transport format: FP32 slice pairs (Re s, Re s+1, Im s, Im s+1), FP64
    (Re, Im) per slice)."""
    num = den = 0.0
    for mu in range(4):
        for face in (0, 1):
            a = x32.halo_pack(mu, face).view(np.float32).reshape(-1, LS // 2, 2, 2)
            a = a.transpose(0, 1, 3, 2).reshape(-1, LS, 2).astype(np.float64)  # (re/im pairs) -> (slice, re/im)
            b = x64.halo_pack(mu, face).view(np.float64).reshape(-1, LS, 2)
            num += float(np.sum((a - b) ** 2))
            den += float(np.sum(b ** 2))
    return float(np.sqrt(num / den))


def measured_fp64_peak() -> dict | None:
    """FP64 throughput of the GPU, measured here: a cuBLAS DGEMM (8192^3, through torch, which
    is only plumbing for this one number), best of 3 with CUDA events.  The FP64 hopping kernel
    is FP64-pipe bound, so it is reported against this as well as against HBM."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
        n = 8192
        a = torch.randn(n, n, dtype=torch.float64, device="cuda")
        b = torch.randn(n, n, dtype=torch.float64, device="cuda")
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        del a, b
        torch.cuda.empty_cache()
        return {"value": round(2.0 * n ** 3 / best / 1e12, 3), "unit": "TFLOP/s", "how": "cuBLAS DGEMM 8192^3"}
    except Exception:
        return None


def secondary(gb, args, peak) -> dict:
    out = {}
    lat = gb.Lattice.periodic(DIMS, LS)
    V5 = int(np.prod(DIMS)) * LS
    g64 = gb.Gauge(lat, None, gb.F64, seed=11)
    g32 = gb.Gauge(lat, None, gb.F32, seed=11)
    g16 = gb.Gauge(lat, None, gb.F16, seed=11)
    x64 = gb.Field(lat, gb.F64).gaussian(21)
    y64 = gb.Field(lat, gb.F64)
    x32, y32 = gb.Field(lat, gb.F32), gb.Field(lat, gb.F32)
    x32.copy_from(x64)
    x16, y16 = gb.Field(lat, gb.F16), gb.Field(lat, gb.F16)
    x16.copy_from(x64)
    steps = 200
    for name, g, x, y, sp, gp, dag in (("dhop_f64_16^4x16", g64, x64, y64, 0, 0, 0),
                                       ("dhopdag_f32_16^4x16", g32, x32, y32, 1, 1, 1),
                                       ("dhop_f16_16^4x16", g16, x16, y16, 2, 2, 0)):
        gb.tune_dhop(g, y, x, dag)
        n = steps if sp != 0 else 40
        ms, _ = time_dhop(gb, g, [(y, x)], n, 5, dag)
        t = ms / n / 1e3
        ref = gb.Field(lat, gb.F64)
        gb.dhop(g64, ref, x64, dag)
        rec = {"gflops": round(FLOP_PER_SITE * V5 / t / 1e9, 1), "ms": round(t * 1e3, 4),
               "hbm_frac": round(algo_bytes(sp, gp, LS) * V5 / t / 1e9 / peak, 3),
               "rel_err_vs_fp64": 0.0 if sp == 0 else rel_to(gb, lat, y, ref),
               "launch": list(gb.tune_query(g, x))}
        if sp == 0:
            rec["fp64_tflops"] = round(FLOP_PER_SITE * V5 / t / 1e12, 3)
            fp64_peak = measured_fp64_peak()
            if fp64_peak:
                rec["fp64_peak_tflops"] = fp64_peak
                rec["fp64_frac"] = round(rec["fp64_tflops"] / fp64_peak["value"], 3)
            # the same FP64 fields through the double-single form (FP32-pair arithmetic)
            gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_DOUBLE_SINGLE)
            try:
                ms, _ = time_dhop(gb, g, [(y, x)], steps, 5, dag)
                t_ds = ms / steps / 1e3
                rec["double_single"] = {
                    "ms": round(t_ds * 1e3, 4), "gflops": round(FLOP_PER_SITE * V5 / t_ds / 1e9, 1),
                    "hbm_frac": round(algo_bytes(0, 0, LS) * V5 / t_ds / 1e9 / peak, 3),
                    "speedup_vs_fp64": round(t / t_ds, 2), "rel_err_vs_fp64": rel_to(gb, lat, y, ref),
                    "launch": [128, 1, 0]}
            finally:
                gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_NATIVE)
        out[name] = rec
    # even-odd: the hopping term between half lattices and the closed-form D5^-1 (FP32)
    le, lo = lat.checkerboard()
    ge = g32.checkerboard(le)
    xo = gb.Field(lo, gb.F32).pick(x32)
    ye, ze = gb.Field(le, gb.F32), gb.Field(le, gb.F32)
    gb.tune_dhop(g32, y32, x32)
    for _ in range(5):
        gb.dhop_eo(ge, ye, xo)
    gb.synchronize()
    tm = gb.Timer()
    tm.start()
    for _ in range(steps):
        gb.dhop_eo(ge, ye, xo)
    t = tm.stop() / steps / 1e3
    gb.dwf_m5inv(ze, ye, 1.8, 0.01)
    gb.synchronize()
    tm.start()
    for _ in range(steps):
        gb.dwf_m5inv(ze, ye, 1.8, 0.01)
    t5 = tm.stop() / steps / 1e3
    # FP64 references on the same input values
    ge64 = g64.checkerboard(le)
    xo64, ye64, yy64, ze64 = gb.Field(lo, gb.F64), gb.Field(le, gb.F64), gb.Field(le, gb.F64), gb.Field(le, gb.F64)
    xo64.copy_from(xo)
    gb.dhop_eo(ge, ye, xo)
    gb.dhop_eo(ge64, ye64, xo64)
    eo_err = rel_to(gb, le, ye, ye64)
    yy64.copy_from(ye)
    gb.dwf_m5inv(ze, ye, 1.8, 0.01)
    gb.dwf_m5inv(ze64, yy64, 1.8, 0.01)
    m5_err = rel_to(gb, le, ze, ze64)
    out["dhop_eo_f32_16^4x16"] = {
        "gflops": round(FLOP_PER_SITE * V5 / 2 / t / 1e9, 1), "ms": round(t * 1e3, 4),
        "hbm_frac": round(algo_bytes(1, 1, LS) * V5 / 2 / t / 1e9 / peak, 3), "launch": list(gb.tune_query(g32, x32)),
        "rel_err_vs_fp64": eo_err,
        "m5inv_ms": round(t5 * 1e3, 4), "m5inv_hbm_frac": round(2 * 96 * V5 / 2 / t5 / 1e9 / peak, 3),
        "m5inv_rel_err_vs_fp64": m5_err}
    del ge, xo, ye, ze, ge64, xo64, ye64, yy64, ze64, le, lo
    # Mobius (b = 1.5, c = 0.5): M = Mooee - 1/2 Dhop A(b, c) is one 5th-dimension pass and the
    # hopping pass with the Mooee epilogue; the 5th-dimension pass alone is HBM bound (one FP32
    # spinor read and one written per 5D site)
    t32 = gb.Field(lat, gb.F32)

    def per_call(fn):
        for _ in range(5):
            fn()
        gb.synchronize()
        tm.start()
        for _ in range(steps):
            fn()
        return tm.stop() / steps / 1e3

    tmob = per_call(lambda: gb.mobius_m(g32, y32, t32, x32, 1.5, 0.5, 1.8, 0.01))
    # the same operator in FP64 on the same input (x64 holds the values x32 was rounded from;
    # the FP64 reference takes x32's own values)
    xr, yr, tr = gb.Field(lat, gb.F64), gb.Field(lat, gb.F64), gb.Field(lat, gb.F64)
    xr.copy_from(x32)
    gb.mobius_m(g32, y32, t32, x32, 1.5, 0.5, 1.8, 0.01)
    gb.mobius_m(g64, yr, tr, xr, 1.5, 0.5, 1.8, 0.01)
    mob_err = rel_to(gb, lat, y32, yr)
    tmobd = per_call(lambda: gb.mobius_m(g32, y32, t32, x32, 1.5, 0.5, 1.8, 0.01, 1))
    gb.mobius_m(g32, y32, t32, x32, 1.5, 0.5, 1.8, 0.01, 1)
    gb.mobius_m(g64, yr, tr, xr, 1.5, 0.5, 1.8, 0.01, 1)
    mobd_err = rel_to(gb, lat, y32, yr)
    tsham = per_call(lambda: gb.dwf_m(g32, y32, x32, 1.8, 0.01))
    gb.dwf_m(g64, yr, xr, 1.8, 0.01)
    gb.dwf_m(g32, y32, x32, 1.8, 0.01)
    sham_err = rel_to(gb, lat, y32, yr)
    tm5d = per_call(lambda: gb.mobius_mooee(t32, x32, 1.5, 0.5, 1.8, 0.01))
    out["mobius_m_f32_16^4x16"] = {
        "ms": round(tmob * 1e3, 4), "mdag_ms": round(tmobd * 1e3, 4), "mdag_rel_err_vs_fp64": mobd_err,
        "mdag_form": "one hopping pass, A(b,c)^dag in the epilogue", "shamir_m_ms": round(tsham * 1e3, 4),
        "m5d_ms": round(tm5d * 1e3, 4), "m5d_hbm_frac": round(2 * 96 * V5 / tm5d / 1e9 / peak, 3),
        "rel_err_vs_fp64": mob_err, "shamir_m_rel_err_vs_fp64": sham_err,
        "b": 1.5, "c": 0.5, "M5": 1.8, "mf": 0.01}
    del t32, tr
    # halo packing for a domain decomposition: the 8 faces' projected half spinors into device
    # buffers (allocated through torch, plumbing only); HBM bytes = every face spinor read once,
    # half of it written.  Four source fields rotate so the faces read (4 x 50 MB) exceed L2.
    try:
        import torch
        bufs = [torch.empty(x32.halo_bytes(mu), dtype=torch.uint8, device="cuda") for mu in range(4) for _ in (0, 1)]
        ptrs = [b.data_ptr() for b in bufs]
        srcs = [x32] + [gb.Field(lat, gb.F32) for _ in range(3)]
        for q in srcs[1:]:
            q.copy_from(x32)
        rot = [0]

        def pack_all():
            srcs[rot[0] % 4].halo_pack_all(ptrs)
            rot[0] += 1

        thalo = per_call(pack_all)
        face5 = sum(int(np.prod(DIMS)) // DIMS[mu] for mu in range(4)) * 2 * LS
        out["halo_pack_f32_16^4x16_8faces"] = {
            "us": round(thalo * 1e6, 2), "face_sites5": face5, "bytes": face5 * (96 + 48),
            "hbm_frac": round(face5 * (96 + 48) / thalo / 1e9 / peak, 3), "launches": 1,
            "rel_err_vs_fp64": halo_rel_err(x32, xr),
            "l2": "four source fields rotate: 200 MB of faces read vs 129 MB L2"}
        del bufs, srcs
    except ImportError:
        pass
    del g64, g32, g16, x64, y64, x32, y32, x16, y16, xr, yr, lat
    if not args.quick:
        out["multi_rhs_24^4x12_k12"] = bench_mrhs(gb, peak)
        out["batch_64"] = bench_batch(gb, peak)
        out["batch_64_rhs_1_2_4"] = bench_batch(gb, peak, (1, 2, 4), seed=2025)
        out["cg_32^4x16"] = bench_cg(gb, args)
    return out


def bench_mrhs(gb, peak) -> dict:
    dims, Ls, k = (24, 24, 24, 24), 12, 12
    lat = gb.Lattice.periodic(dims, Ls)
    V5 = int(np.prod(dims)) * Ls
    g = gb.Gauge(lat, None, gb.F32, seed=5)
    X, Y = gb.Field(lat, gb.F32, k), gb.Field(lat, gb.F32, k)
    for r in range(k):
        X.gaussian(100 + r, r)
    gb.tune_dhop(g, Y, X)
    ms_multi, _ = time_dhop(gb, g, [(Y, X)], 10, 2)
    t_multi = ms_multi / 10 / 1e3
    x1, y1 = gb.Field(lat, gb.F32), gb.Field(lat, gb.F32)
    gb.tune_dhop(g, y1, x1)
    # 12 single-RHS launches per step
    singles = []
    for r in range(k):
        s = gb.Field(lat, gb.F32)
        s.gaussian(100 + r, 0)
        singles.append(s)
    outs = [gb.Field(lat, gb.F32) for _ in range(2)]
    ms_single, _ = time_dhop(gb, g, [(outs[r % 2], singles[r]) for r in range(k)], 10 * k, k)
    t_single = ms_single / 10 / 1e3
    # error of the 12-RHS result against single launches (rhs 0), through host export, and of
    # all 12 against the FP64 hopping term of the same sources
    gb.dhop(g, Y, X)
    gb.dhop(g, y1, singles[0])
    err = float(np.linalg.norm(Y.numpy(0) - y1.numpy()) / np.linalg.norm(y1.numpy()))
    del singles, outs
    g64 = gb.Gauge(lat, None, gb.F64, seed=5)
    X64, Y64 = gb.Field(lat, gb.F64, k), gb.Field(lat, gb.F64, k)
    X64.copy_from(X)
    gb.dhop(g64, Y64, X64)
    err64 = rel_to(gb, lat, Y, Y64)
    del g64, X64, Y64
    per_src_multi = FLOP_PER_SITE * V5 * k / t_multi / 1e9
    per_src_single = FLOP_PER_SITE * V5 * k / t_single / 1e9
    return {"gflops_12rhs": round(per_src_multi, 1), "gflops_12x1rhs": round(per_src_single, 1),
            "per_source_speedup": round(per_src_multi / per_src_single, 3),
            "byte_model_ceiling": round(algo_bytes(1, 1, Ls, 1) / algo_bytes(1, 1, Ls, k), 3),
            "hbm_frac_12rhs": round(algo_bytes(1, 1, Ls, k) * V5 * k / t_multi / 1e9 / peak, 3),
            "rel_err_vs_single": err, "rel_err_vs_fp64": err64, "launch": list(gb.tune_query(g, X)),
            "tile_split": gb.tune_split(g, X), "t_brick": gb.tune_brick(g, X),
            "single_rhs_launch": list(gb.tune_query(g, x1)) + [gb.tune_split(g, x1), gb.tune_brick(g, x1)]}


def bench_batch(gb, peak, nrhs_choices=(1,), seed=2024, vols=(8, 12, 16, 20, 24)) -> dict:
    """64 instances in one persistent launch replayed from a CUDA graph: 4D volumes uniform over
    {8^4 .. 24^4}, Ls over {8, 12, 16}, FP32 or FP16 storage, right-hand sides from
    nrhs_choices; against the same instances as 64 separate launches, each on its own
    autotuned shape."""
    rng = np.random.default_rng(seed)
    vols = list(vols)
    keep, G, O, I, spec = [], [], [], [], []
    flops = 0
    sites5 = 0
    nbytes = 0.0
    for k in range(64):
        L = int(rng.choice(vols))
        Ls = int(rng.choice([8, 12, 16]))
        prec = gb.F32 if rng.random() < 0.5 else gb.F16
        nrhs = int(rng.choice(nrhs_choices))
        lat = gb.Lattice.periodic((L, L, L, L), Ls)
        g = gb.Gauge(lat, None, prec, seed=1000 + k)
        x = gb.Field(lat, prec, nrhs)
        for r in range(nrhs):
            x.gaussian(2000 + 97 * k + r, r)
        y = gb.Field(lat, prec, nrhs)
        keep.append(lat)
        G.append(g)
        O.append(y)
        I.append(x)
        spec.append((L, Ls, prec, nrhs))
        flops += FLOP_PER_SITE * L ** 4 * Ls * nrhs
        sites5 += L ** 4 * Ls * nrhs
        sp = 1 if prec == gb.F32 else 2
        nbytes += algo_bytes(sp, sp, Ls, nrhs) * L ** 4 * Ls * nrhs
    t0 = time.perf_counter()
    b = gb.Batch(G, O, I)
    tune_s = time.perf_counter() - t0
    for _ in range(3):
        b.run()
    gb.synchronize()
    t = gb.Timer()
    reps = 10
    t.start()
    for _ in range(reps):
        b.run()
    ms = t.stop() / reps
    # the same instances as 64 separate launches, each (precision, Ls*nrhs) on its tuned shape
    tuned = set()
    for g, y, x, (L, Ls, prec, nrhs) in zip(G, O, I, spec):
        if (prec, Ls * nrhs) not in tuned:
            gb.tune_dhop(g, y, x)
            tuned.add((prec, Ls * nrhs))
    for g, y, x in zip(G, O, I):
        gb.dhop(g, y, x)
    gb.synchronize()
    t.start()
    for _ in range(reps):
        for g, y, x in zip(G, O, I):
            gb.dhop(g, y, x)
    ms_sep = t.stop() / reps
    info = b.info()
    # every instance against the FP64 hopping term of its own input values
    b.run()
    gb.synchronize()
    errs = {gb.F32: 0.0, gb.F16: 0.0}
    for k, (L, Ls, prec, nrhs) in enumerate(spec):
        g64 = gb.Gauge(keep[k], None, gb.F64, seed=1000 + k)
        x64, y64 = gb.Field(keep[k], gb.F64, nrhs), gb.Field(keep[k], gb.F64, nrhs)
        x64.copy_from(I[k])
        gb.dhop(g64, y64, x64)
        errs[prec] = max(errs[prec], rel_to(gb, keep[k], O[k], y64))
        del g64, x64, y64
    return {"instances": 64, "rhs_choices": list(nrhs_choices), "sites5": sites5,
            "gflops": round(flops / (ms / 1e3) / 1e9, 1),
            "ms_per_replay": round(ms, 3), "ms_64_separate_launches": round(ms_sep, 3),
            "speedup_vs_separate": round(ms_sep / ms, 3),
            "hbm_frac": round(nbytes / (ms / 1e3) / 1e9 / peak, 3), "algorithmic_bytes": int(nbytes),
            "rel_err_vs_fp64": {"fp32_max": errs[gb.F32], "fp16_max": errs[gb.F16]},
            "graph": info["graph"], "ctas": info["ctas"], "threads": info["threads"],
            "shape": {"spt_f32": info["spt_f32"], "spt_f16": info["spt_f16"], "tile_split": info["tile_split"]},
            "tune_seconds": round(tune_s, 2)}


def bench_cg(gb, args) -> dict:
    """Time to a 1e-10 true residual, plain (FP32 operator, FP64 vectors) against mixed
    (FP16 or FP32 operator, reliable updates), on M^dag M x = b over the full lattice and on
    M x = b through the even-odd Schur complement.  Each mode runs at the reliable-update
    threshold delta measured best for it on this problem (FP16 drifts fastest: 0.03 on the full
    lattice, 0.02 through the Schur complement; the FP32 operator holds to 1e-4).  The FP16 runs keep the iterated residual in FP16 as well
    (sloppy_residual = 1: same iterations and reliable updates, 6 % less time than an FP32 r)."""
    dims, Ls = ((32, 32, 32, 32), 16) if not args.cg_small else ((16, 16, 16, 16), 16)
    M5, mf = 1.8, 0.01
    lat = gb.Lattice.periodic(dims, Ls)
    le, lo = lat.checkerboard()
    g64 = gb.Gauge(lat, None, gb.F64, seed=77)
    g32 = gb.Gauge(lat, None, gb.F32, seed=77)
    g16 = gb.Gauge(lat, None, gb.F16, seed=77)
    m_shapes = {}
    # the solvers' FP64 operator (true residuals) runs double-single: tune that form's shapes
    gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_DOUBLE_SINGLE)
    try:
        x, y = gb.Field(lat, gb.F64).gaussian(1), gb.Field(lat, gb.F64)
        gb.tune_dhop(g64, y, x)
        m_shapes["fp64_double_single"] = {"dhop": list(gb.tune_query_ds(g64, x, 0)),
                                          "m": list(gb.tune_query_ds(g64, x, 1)),
                                          "fields": "CTAs per SM of the register cap, t-brick"}
        del x, y
    finally:
        gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_NATIVE)
    for g, sp, tag in ((g32, gb.F32, "fp32"), (g16, gb.F16, "fp16")):
        x, y = gb.Field(lat, sp).gaussian(1), gb.Field(lat, sp)
        gb.tune_dhop(g, y, x)
        m_shapes[tag] = {"dhop": list(gb.tune_query(g, x)) + [gb.tune_split(g, x), gb.tune_brick(g, x)],
                         "m": list(gb.tune_query_m(g, x)),
                         "cg_step_r_fp64" if sp == gb.F32 else "cg_step_r_fp16":
                             list(gb.tune_query_cg(g, x, gb.F64 if sp == gb.F32 else gb.F16)),
                         "cg_step_r_fp32": list(gb.tune_query_cg(g, x, gb.F32))}
        del x, y
    G64 = (g64.checkerboard(le), g64.checkerboard(lo))
    G32 = (g32.checkerboard(le), g32.checkerboard(lo))
    G16 = (g16.checkerboard(le), g16.checkerboard(lo))
    for G, sp, tag in ((G32, gb.F32, "fp32"), (G16, gb.F16, "fp16")):
        # the even-odd operator tunes on its own operands (gauge and output on the even half)
        xo, ye = gb.Field(lo, sp).gaussian(1), gb.Field(le, sp)
        gb.tune_dhop(G[0], ye, xo)
        m_shapes[tag]["eo_hop"] = list(gb.tune_query(G[0], xo)) + [gb.tune_split(G[0], xo), 1]
        m_shapes[tag]["eo_schur"] = list(gb.tune_query_m(G[0], xo))
        del xo, ye
    b = gb.Field(lat, gb.F64).gaussian(78)
    res = {"lattice": f"{'x'.join(map(str, dims))} x Ls={Ls}", "M5": M5, "mf": mf, "tol": 1e-10,
           "full": "CG on M^dag M x = b; true_residual = |b - M^dag M x| / |b|",
           "eo": "M x = b by CG on the odd Schur normal system (tol on its true residual); "
                 "true_residual = |b - M x| / |b| after reconstruction",
           "launch": m_shapes, "launch_fields": "threads, slices/thread, form, stages, tile split, t-brick"}
    it = args.cg_max_iter
    runs = (
        ("full_plain_fp32_fp64res", 1e-4, lambda x, d: gb.cg_solve(g64, x, b, M5, mf, gb.CG_PLAIN, max_iter=it, delta=d,
                                                                   g32=g32)),
        ("full_mixed_fp16", 0.03, lambda x, d: gb.cg_solve(g64, x, b, M5, mf, gb.CG_MIXED, max_iter=it, delta=d, g32=g32,
                                                          gsloppy=g16, sloppy_prec=gb.F16, sloppy_residual=1)),
        ("full_mixed_fp32", 1e-4, lambda x, d: gb.cg_solve(g64, x, b, M5, mf, gb.CG_MIXED, max_iter=it, delta=d,
                                                           g32=g32, gsloppy=g32, sloppy_prec=gb.F32)),
        ("eo_plain_fp32_fp64res", 1e-4, lambda x, d: gb.cg_solve_eo(G64, x, b, M5, mf, gb.CG_PLAIN, max_iter=it,
                                                                    delta=d, g32=G32)),
        ("eo_mixed_fp16", 0.02, lambda x, d: gb.cg_solve_eo(G64, x, b, M5, mf, gb.CG_MIXED, max_iter=it, delta=d,
                                                            g32=G32, gsloppy=G16, sloppy_prec=gb.F16,
                                                            sloppy_residual=1)),
        ("eo_mixed_fp32", 1e-4, lambda x, d: gb.cg_solve_eo(G64, x, b, M5, mf, gb.CG_MIXED, max_iter=it, delta=d,
                                                            g32=G32, gsloppy=G32, sloppy_prec=gb.F32)),
    )
    for name, delta, fn in runs:
        x = gb.Field(lat, gb.F64)
        try:
            st = fn(x, delta)
            res[name] = {k: (round(v, 6) if isinstance(v, float) and k != "true_residual" else v)
                         for k, v in st.items()}
            res[name]["delta"] = delta
        except gb.GbdwError as e:
            res[name] = {"error": str(e)}
        del x
    for pre in ("full", "eo"):
        plain = res.get(f"{pre}_plain_fp32_fp64res", {})
        for sp in ("fp16", "fp32"):
            mixed = res.get(f"{pre}_mixed_{sp}", {})
            if "seconds" in plain and "seconds" in mixed:
                res[f"speedup_{pre}_mixed_{sp}_vs_plain"] = round(plain["seconds"] / mixed["seconds"], 3)
    if "seconds" in res.get("full_plain_fp32_fp64res", {}) and "seconds" in res.get("eo_mixed_fp32", {}):
        res["note"] = "full and eo solve different systems (M^dag M x = b vs M x = b); compare within a row"
    return res


def run_ours(args, D: Dist) -> dict | None:
    import gridbench_gb300 as gb
    gb.load()
    if not gb.device_available():
        raise SystemExit("bench.py: no CUDA device visible (" + gb.load().gbdw_last_error().decode() + ")")
    peak, peak_src = measured_peak_hbm()
    V5 = int(np.prod(DIMS)) * LS
    lat = gb.Lattice.periodic(DIMS, LS)
    U = gb.generate_gauge(DIMS)
    g = gb.Gauge(lat, U, gb.F32)
    phiA = gb.generate_fermion(DIMS, LS)
    xA = gb.Field(lat, gb.F32).load(phiA)
    xB = gb.Field(lat, gb.F32).load(gb.generate_fermion(DIMS, LS, 1, (9, 10, 11, 12)))
    yA, yB = gb.Field(lat, gb.F32), gb.Field(lat, gb.F32)
    if args.tune_load:
        gb.tune_load(args.tune_load)
    else:
        gb.tune_dhop(g, yA, xA)
    if args.tune_save:
        gb.tune_save(args.tune_save)
    cfg = gb.tune_query(g, xA)
    pairs = [(yA, xA), (yB, xB)]
    clocks = Clocks()
    clocks.start()
    for i in range(args.warmup):
        y, x = pairs[i % 2]
        gb.dhop(g, y, x)
    gb.synchronize()
    D.barrier()
    clocks.mark("t0")
    ms, launches = time_dhop(gb, g, pairs, args.steps, 0)
    clocks.mark("t1")
    clk = clocks.stop()
    ms = D.max(ms)
    t_step = ms / args.steps / 1e3
    flops_step = FLOP_PER_SITE * V5
    value = D.world * flops_step / t_step / 1e9
    bytes_launch = algo_bytes(1, 1, LS) * V5
    achieved = bytes_launch / t_step / 1e9
    traffic = ncu_traffic("dhop_f32_16^4x16")

    # end to end through the public API: pinned host input -> device -> Dhop -> pinned host
    # output, every step.  Steps rotate over three library streams with their own fields and
    # host buffers, so one step's result write-back overlaps the next steps' input reads (the
    # host link is full duplex); each step still moves its whole input in and result out.
    n = V5 * 24
    NS = 3  # streams: a stream's next input copy queues behind its own previous write-back
    hins = [gb.PinnedArray(n, np.float32) for _ in range(NS)]
    houts = [gb.PinnedArray(n, np.float32) for _ in range(NS)]
    for h in hins:
        h.array[:] = phiA
    streams = [gb.Stream() for _ in range(NS)]
    epairs = [(xA, yA), (xB, yB), (gb.Field(lat, gb.F32), gb.Field(lat, gb.F32))]

    def e2e_step(i):
        k = i % NS
        with streams[k]:
            x, y = epairs[k]
            x.load(hins[k].array)
            gb.dhop(g, y, x)
            y.export_into(houts[k].array, sync=False)

    e2e_steps = max(2 * NS, min(args.steps, 300)) // NS * NS
    for i in range(2 * NS):
        e2e_step(i)
    for st in streams:
        st.synchronize()
    D.barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        e2e_step(i)
    for st in streams:
        st.synchronize()
    te = D.max(time.perf_counter() - t0) / e2e_steps
    check_out = np.empty(n, np.float32)
    yA.export_into(check_out)
    e2e_ok = bool(all(np.array_equal(check_out, h.array) for h in houts))
    for st in streams:
        st.close()
    e2e = {"value": round(D.world * flops_step / te / 1e9, 2), "unit": "GFLOP/s",
           "h2d_bytes_per_step": int(hins[0].array.nbytes), "d2h_bytes_per_step": int(houts[0].array.nbytes),
           "steps": e2e_steps, "ms_per_step": round(te * 1e3, 4), "results_match": e2e_ok,
           "path": "Field.load(pinned FP32 reference layout) -> dhop -> Field.export_into(pinned, async); "
                   f"steps rotate over {NS} streams"}

    # relative error of this FP32 result against the FP64 kernel on the same input
    g64 = gb.Gauge(lat, U, gb.F64)
    x64, y64 = gb.Field(lat, gb.F64).load(phiA), gb.Field(lat, gb.F64)
    gb.dhop(g64, y64, x64)
    gb.dhop(g, yA, xA)
    rel = rel_to(gb, lat, yA, y64)
    del g64, x64, y64

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GFLOP/s", "n_gpus": D.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic: seeded random SU(3) links (Gaussian -> Gram-Schmidt -> det 1), N(0,1) fermion",
        "config": dict(CONFIG),
        "parallelism": "replicas" if D.world > 1 else "single",
        "launch": {"threads": cfg[0], "slices_per_thread": cfg[1],
                   "form": {0: "direct", 1: "tma-staged (CTA ring)", 2: "tma-staged (warp rings)",
                            3: "direct (Ls=16 specialised)", 4: "direct (Ls=16, 2^4 site blocks)"}[cfg[2]],
                   "stages": cfg[3], "tile_split": gb.tune_split(g, xA), "t_brick": gb.tune_brick(g, xA)},
        "rel_err_vs_fp64": rel,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                     else "fallback 6.8 TB/s",
                     "algorithmic_bytes_per_launch": int(bytes_launch),
                     "bytes_per_site": algo_bytes(1, 1, LS)},
        "e2e": e2e,
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    if D.rank == 0 and D.world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(DIMS, LS, args.cpu_seconds)
    if not args.no_secondary:
        line["secondary"] = secondary(gb, args, peak)
    return line if D.rank == 0 else None


# ------------------------------------------------------------------ reference arm
def run_reference(args, D: Dist) -> dict | None:
    """The reference's algorithm on the host CPU: the oracle port of dslash_simple.h (the
    reference's own kernels are x86-only and its tree is not present on the GPU host), all
    host threads, each step a bounded sample of the 16^4 x Ls=16 FP32 workload.  Inputs come
    from the oracle's own generator: this arm never loads the product library.  Like our arm
    it alternates two in/out pairs."""
    if D.rank != 0:
        return None
    import oracle
    U = oracle.generate_gauge(DIMS).astype(np.float32)
    phis = [oracle.generate_fermion(DIMS, LS).astype(np.float32),
            oracle.generate_fermion(DIMS, LS, 1, (9, 10, 11, 12)).astype(np.float32)]
    nbr, prm, nsite = oracle.generate_table(DIMS, LS)
    outs = [np.zeros_like(phis[0]) for _ in range(2)]
    oracle.dslash_sites(U, phis[0], outs[0], nbr, 0, nsite, LS)
    t = time.perf_counter()
    oracle.dslash_sites(U, phis[0], outs[0], nbr, 0, nsite, LS)
    t_full = time.perf_counter() - t
    budget = args.ref_seconds
    per_step = budget / max(1, args.steps + args.warmup)
    frac = min(1.0, per_step / t_full)
    sample = max(64, int(nsite * frac))
    sample = min(sample, nsite)
    for i in range(args.warmup):
        oracle.dslash_sites(U, phis[i % 2], outs[i % 2], nbr, 0, sample, LS)
    t = time.perf_counter()
    for i in range(args.steps):
        s0 = (i * sample) % (nsite - sample + 1)
        oracle.dslash_sites(U, phis[i % 2], outs[i % 2], nbr, s0, s0 + sample, LS)
    dt = time.perf_counter() - t
    value = FLOP_PER_SITE * sample * LS * args.steps / dt / 1e9
    desc = (f"each step: {sample} of {nsite} 4D sites (x Ls={LS}) of the 16^4 FP32 lattice, "
            f"{args.steps} steps in {dt:.2f} s")
    return {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GFLOP/s", "n_gpus": D.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic: seeded random SU(3) links (Gaussian -> Gram-Schmidt -> det 1), N(0,1) fermion",
            "config": dict(CONFIG),
            "cpu_baseline": {"value": round(value, 3), "unit": "GFLOP/s", "cores": oracle.threads(), "kind": "port",
                             "sample": desc, "why_port": WHY_PORT},
            "e2e": {"value": round(value, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


ONLY = {  # name -> (dims, Ls, spinor precision, gauge precision, dag[, right-hand sides])
    "dhop_f32": (DIMS, LS, 1, 1, 0), "dhopdag_f32": (DIMS, LS, 1, 1, 1), "dhop_f64": (DIMS, LS, 0, 0, 0),
    "dhop_f16": (DIMS, LS, 2, 2, 0), "dhop_bf16": (DIMS, LS, 2, 3, 0),
    # the 12-RHS kernel on a lattice small enough for a full profile (2 x 0.9 GB fields)
    "dhop_f32_12rhs_16x12": (DIMS, 12, 1, 1, 0, 12),
    # FP64 fields through the double-single form, at the shape its tuner picks at 16^4 x 16
    # (registers capped for four CTAs per SM, natural order)
    "dhop_f64ds": (DIMS, LS, 0, 0, 0),
}


CG_ONLY = ("cg_full_plain", "cg_full_mixed16", "cg_eo_plain", "cg_eo_mixed16", "cg32")


def run_cg_only(args) -> dict:
    """One CG solve (16^4 x Ls=16, tol 1e-10), nothing else: the command its launch list is
    captured with."""
    import gridbench_gb300 as gb
    if args.only == "cg32":
        return {"workload": "cg32", **bench_cg(gb, args)}
    dims, Ls, M5, mf = (16, 16, 16, 16), 16, 1.8, 0.01
    lat = gb.Lattice.periodic(dims, Ls)
    g64, g32, g16 = (gb.Gauge(lat, None, p, seed=77) for p in (gb.F64, gb.F32, gb.F16))
    b = gb.Field(lat, gb.F64).gaussian(78)
    x = gb.Field(lat, gb.F64)
    # the shapes the tuner picks on a GB300 for these extents, pinned (a profiler would reorder it)
    gb.tune_set(g32, gb.Field(lat, gb.F32), 64, 2, 2, 2)
    gb.tune_set(g16, gb.Field(lat, gb.F16), 64, 2, 3, 4)
    if args.only.startswith("cg_eo"):
        le, lo = lat.checkerboard()
        G = [(g.checkerboard(le), g.checkerboard(lo)) for g in (g64, g32, g16)]
        if args.only == "cg_eo_plain":
            st = gb.cg_solve_eo(G[0], x, b, M5, mf, gb.CG_PLAIN, delta=1e-4, g32=G[1])
        else:
            st = gb.cg_solve_eo(G[0], x, b, M5, mf, gb.CG_MIXED, delta=0.02, g32=G[1], gsloppy=G[2],
                                sloppy_prec=gb.F16, sloppy_residual=1)
    elif args.only == "cg_full_plain":
        st = gb.cg_solve(g64, x, b, M5, mf, gb.CG_PLAIN, delta=1e-4, g32=g32)
    else:
        st = gb.cg_solve(g64, x, b, M5, mf, gb.CG_MIXED, delta=0.03, g32=g32, gsloppy=g16, sloppy_prec=gb.F16,
                         sloppy_residual=1)
    return {"workload": args.only, "lattice": list(dims), "Ls": Ls, **st}


def run_only(args) -> dict:
    """One hopping-term workload, nothing else: the command profiles are captured with.
    --shape threads,slices,form,stages pins the launch shape (form 0 direct, 1 TMA-staged CTA
    ring, 2 TMA-staged warp rings, 3 direct specialised for Ls=16);
    without it the autotuner picks."""
    import gridbench_gb300 as gb
    dims, Ls, sp, gp, dag = ONLY[args.only][:5]
    k = ONLY[args.only][5] if len(ONLY[args.only]) > 5 else 1
    lat = gb.Lattice.periodic(dims, Ls)
    g = gb.Gauge(lat, None, gp, seed=11)
    xs = [gb.Field(lat, sp, k) for _ in range(2)]
    for i, x in enumerate(xs):
        for r in range(k):
            x.gaussian(21 + i + 2 * r, r)
    ys = [gb.Field(lat, sp, k) for _ in range(2)]
    if args.only == "dhop_f64ds":
        gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_DOUBLE_SINGLE)
        gb.tune_set_ds(g, xs[0], 0, 4, 1)
    elif args.shape:
        th, spt, form, st = (int(v) for v in args.shape.split(","))
        gb.tune_set(g, xs[0], th, spt, form, st)
    else:
        gb.tune_dhop(g, ys[0], xs[0], dag)
    ms, launches = time_dhop(gb, g, list(zip(ys, xs)), args.steps, args.warmup, dag)
    gb.synchronize()
    V5 = int(np.prod(dims)) * Ls * k
    t = ms / args.steps / 1e3
    peak, _ = measured_peak_hbm()
    return {"workload": args.only, "lattice": list(dims), "Ls": Ls, "rhs": k, "steps": args.steps,
            "us_per_launch": round(t * 1e6, 3), "gflops": round(FLOP_PER_SITE * V5 / t / 1e9, 1),
            "hbm_frac": round(algo_bytes(sp, gp, Ls, k) * V5 / t / 1e9 / peak, 4),
            "shape": list(gb.tune_query(g, xs[0])), "gpu_launches": int(launches)}


AUX_ONLY = ("mobius_m", "mobius_mdag", "halo_pack", "batch", "batch_rhs", "batch_small", "mrhs")


def run_aux_only(args) -> dict:
    """The Mobius operator (b = 1.5, c = 0.5, M5 = 1.8, mf = 0.01) or the one-launch pack of all
    eight halo faces, FP32 16^4 x 16, or one of the 64-instance batches, nothing else (for
    profiling)."""
    import gridbench_gb300 as gb
    if args.only == "mrhs":
        peak, _ = measured_peak_hbm()
        return {"workload": "multi_rhs_24^4x12_k12", **bench_mrhs(gb, peak)}
    if args.only.startswith("batch"):
        peak, _ = measured_peak_hbm()
        if args.only == "batch":
            res = bench_batch(gb, peak)
        elif args.only == "batch_rhs":
            res = bench_batch(gb, peak, (1, 2, 4), seed=2025)
        else:  # 64 instances of at most 12^4 (about 1 GB on the device): the profiling case
            res = bench_batch(gb, peak, vols=(8, 12))
        return {"workload": args.only, **res}
    lat = gb.Lattice.periodic(DIMS, LS)
    g = gb.Gauge(lat, None, gb.F32, seed=11)
    xs = [gb.Field(lat, gb.F32).gaussian(21 + i) for i in range(4)]
    y, t = gb.Field(lat, gb.F32), gb.Field(lat, gb.F32)
    if args.only.startswith("mobius_m"):
        if args.shape:
            gb.tune_set(g, xs[0], *(int(v) for v in args.shape.split(",")))
        else:
            gb.tune_dhop(g, y, xs[0])
        dag = 1 if args.only == "mobius_mdag" else 0
        fn = lambda k: gb.mobius_m(g, y, t, xs[k % 2], 1.5, 0.5, 1.8, 0.01, dag)  # noqa: E731
    else:
        import torch
        bufs = [torch.empty(xs[0].halo_bytes(k // 2), dtype=torch.uint8, device="cuda") for k in range(8)]
        ptrs = [b.data_ptr() for b in bufs]
        fn = lambda k: xs[k % 4].halo_pack_all(ptrs)  # noqa: E731
    for k in range(args.warmup):
        fn(k)
    gb.synchronize()
    tm = gb.Timer()
    n0 = gb.launch_count()
    tm.start()
    for k in range(args.steps):
        fn(k)
    ms = tm.stop()
    return {"workload": args.only, "lattice": list(DIMS), "Ls": LS, "steps": args.steps,
            "us_per_call": round(ms / args.steps * 1e3, 3), "gpu_launches": int(gb.launch_count() - n0)}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--quick", action="store_true", help="skip the 12-RHS, batch and CG secondaries")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-seconds", type=float, default=30.0)
    ap.add_argument("--cg-small", action="store_true", help="CG secondary on 16^4 x 16 instead of 32^4 x 16")
    ap.add_argument("--cg-max-iter", type=int, default=20000)
    ap.add_argument("--only", choices=sorted(ONLY) + list(CG_ONLY) + list(AUX_ONLY),
                    help="one hopping-term workload, or one CG solve at 16^4 x 16, only (for profiling)")
    ap.add_argument("--shape", help="with --only: threads,slices_per_thread,form,stages")
    ap.add_argument("--tune-save", help="write the headline kernel's tuned shapes to this JSON file")
    ap.add_argument("--tune-load", help="take the headline kernel's shapes from this JSON file instead of tuning "
                                        "(a profiler serialises launches, which changes the tuner's ranking)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.only:
        run = run_cg_only if args.only in CG_ONLY else run_aux_only if args.only in AUX_ONLY else run_only
        print(json.dumps(run(args)), flush=True)
        return
    D = Dist()
    try:
        line = run_reference(args, D) if args.impl == "reference" else run_ours(args, D)
        if line is not None:
            print(json.dumps(line), flush=True)
    finally:
        D.close()


if __name__ == "__main__":
    main()

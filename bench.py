#!/usr/bin/env python
"""Benchmark of the cutoff-pair engine on GB300: within-cutoff pairs per second.

Workload (one "step" = cell-list build + pair map over the whole system):
  1,048,576 Float32 particles, fcc lattice (64^3 cells x 4) at density 0.8 mapped through the triclinic
  cell a=(L,0,0), b=(0.2L,L,0), c=(0.1L,0.15L,L), Gaussian jitter sigma=0.05, Lennard-Jones
  (sigma=1, eps=1) energy + forces with cutoff 2.5.  Seeded synthetic data (seed 2).
Forms: exact (input-dtype arithmetic, bit-exact pair set) is `value`; the FP32-split form is reported
beside it (for Float32 inputs it is the exact form; `forms.cfg2_f64` runs the same workload with Float64
positions, where the split form does its distance work in FP32).  `e2e` goes through the C ABI with host buffers (H2D of positions and D2H of energy+forces
inside the timed region).  `--impl reference` times the CPU restatement of the reference algorithm
(OpenMP over all host cores) on the same workload.

Multi-GPU: the path is run as independent replicas (one per rank); value = pairs of all ranks / max time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "within-cutoff pairs/s (cell-list build + pair map, LJ energy+forces)"
# DRAM bytes per launch of the headline pair kernel, from the ncu capture recorded beside its summary
TRAFFIC_RECORD = os.path.join(ROOT, "profiles", "k_pairs_lj_forces_f32_fcc1M_triclinic.json")
WORKLOAD = "fcc1M_f32_triclinic_lj_rc2.5"
CUTOFF = 2.5


def make_workload(ncell=64, rho=0.8, jitter=0.05, seed=2):
    """fcc lattice in fractional coordinates mapped through the triclinic cell matrix, plus jitter."""
    n = 4 * ncell ** 3
    L = (n / rho) ** (1.0 / 3.0)
    g = np.stack(np.meshgrid(np.arange(ncell), np.arange(ncell), np.arange(ncell), indexing="ij"), -1).reshape(-1, 3)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    frac = ((g[:, None, :] + basis[None, :, :]).reshape(-1, 3)) / ncell
    M = np.array([[L, 0.2 * L, 0.1 * L], [0.0, L, 0.15 * L], [0.0, 0.0, L]])  # columns a, b, c
    rng = np.random.default_rng(seed)
    x = frac @ M.T + rng.normal(0.0, jitter, (n, 3))
    return x.astype(np.float32), M


def flops_per_pair(cell_size, cutoff, f_op=20.0):
    """Algorithmic flops per within-cutoff pair: 8*R + F_op, R = 27 h^3 / ((4/3) pi rc^3)."""
    R = 27.0 * float(np.prod(cell_size)) / (4.0 / 3.0 * math.pi * cutoff ** 3)
    return 8.0 * R + f_op, R


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [v.strip() for v in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference(x, M, steps, warmup, threads):
    """The reference algorithm on the host cores: the oracle's cell-list build + threaded map."""
    from oracle import oracle as orc
    kw = dict(kind="tri", unitcell=M, cutoff=CUTOFF, dtype=np.float32, nthreads=threads, compensated=False,
              params=[1.0, 1.0, 4.0, 4.0])
    pairs = orc.run("count", x, **{k: v for k, v in kw.items() if k != "params"})["count"]
    for _ in range(warmup):
        orc.run("lj_forces", x, **kw)
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.run("lj_forces", x, **kw)
    dt = time.perf_counter() - t0
    return pairs, dt


def max_over_ranks(value, world, device=None):
    """Replicas: the job's time is the slowest rank's (all_reduce MAX over the process group)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------------------------- other forms
# Algorithmic flops per within-cutoff pair of each operator epilogue (sqrt/div = 1, FMA = 2).
F_OP = {"nl": 1.0, "soft_energy": 4.0, "soft_forces": 15.0, "lj_forces": 20.0, "lj_forces_types": 22.0,
        "lj_adjoint_types": 42.0, "rhist": 11.0}


def candidates_per_hit(h, cutoff, dim=3):
    """R = 27 h^3 / ((4/3) pi rc^3) in 3D, 9 h^2 / (pi rc^2) in 2D, for cell sides h."""
    h = np.asarray(h, np.float64)
    if dim == 3:
        return 27.0 * float(np.prod(h)) / (4.0 / 3.0 * math.pi * cutoff ** 3)
    return 9.0 * float(np.prod(h)) / (math.pi * cutoff ** 2)


def roofline_pairs(F, peak_tflops, bytes_per_pair=0.0, hbm_gbs=None):
    """min(peak_pipe / F, peak_HBM / bytes per pair) in pairs/s."""
    r = peak_tflops * 1e12 / F
    if bytes_per_pair and hbm_gbs:
        r = min(r, hbm_gbs * 1e9 / bytes_per_pair)
    return r


class Plain:
    """One library handle driven through the C ABI with device-resident inputs, on a torch stream."""

    def __init__(self, L, A, dtype, dim, nsets, stream):
        self.L, self.A = L, A
        self.h = C.c_void_p()
        assert L.clm_create(A.CLM_F64 if dtype == np.float64 else A.CLM_F32, dim, nsets, C.byref(self.h)) == 0
        assert L.clm_set_stream(self.h, C.c_void_p(stream.cuda_stream)) == 0
        self.stream = stream

    def box(self, M, kind, cutoff, lcell=1):
        Mf = np.ascontiguousarray(np.asarray(M, np.float64).flatten(order="F"))
        assert self.L.clm_set_box(self.h, Mf.ctypes.data_as(C.POINTER(C.c_double)), kind, cutoff, lcell) == 0

    def step(self, sets, op, p, o):
        L = self.L
        st = 0
        for k, t in enumerate(sets):
            st = st or L.clm_set_positions(self.h, k, C.c_void_p(t.data_ptr()), t.shape[0], 1)
        st = st or L.clm_run(self.h, op, C.byref(p), C.byref(o))
        if st:
            buf = C.create_string_buffer(512)
            L.clm_last_error(self.h, buf, 512)
            raise RuntimeError(f"clm status {st}: {buf.value.decode()}")

    def timed(self, sets, op, p, o, steps, warmup, flush):
        import torch
        for _ in range(warmup):
            self.step(sets, op, p, o)
        torch.cuda.synchronize()
        tot, kern, build = 0.0, [], []
        for _ in range(steps):
            with torch.cuda.stream(self.stream):
                flush.add_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            self.step(sets, op, p, o)
            e1.record(self.stream)
            e1.synchronize()
            tot += e0.elapsed_time(e1)
            bm, mm = C.c_float(), C.c_float()
            self.L.clm_last_timings(self.h, C.byref(bm), C.byref(mm))
            kern.append(mm.value)
            build.append(bm.value)
        return tot / steps, statistics.median(kern), statistics.median(build)

    def count(self, sets):
        o = self.A.Outputs()
        self.step(sets, self.A.OP["count"], self.A.OpParams(), o)
        return int(o.count)

    def cell_size(self):
        cs = np.zeros(3)
        self.L.clm_get_box(self.h, None, cs.ctypes.data, None, None, None, None, None, None)
        return cs

    def close(self):
        self.L.clm_destroy(self.h)


def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def measure_forms(pkg, L, A, dev, stream, flush, peaks, which, steps, warmup):
    """The other configurations of the metric: plain FP64 box (neighbour list, soft energy, forces), the
    batched form, the adjoint form and the two-set radial histogram, each exact and FP32-split."""
    import torch
    W = pkg.workloads
    out = {}
    p32, p64, hbm = peaks["fp32_tflops"], peaks["fp64_tflops"], peaks["hbm_gbs"]

    def frac_entry(pairs, ms, F, peak, bpp=0.0):
        v = pairs / (ms * 1e-3)
        roof = roofline_pairs(F, peak, bpp, hbm)
        return {"pairs_per_s": v, "kernel_ms": ms, "roofline_pairs_per_s": roof, "frac": v / roof}

    def form_entry(pairs, ms, F, split, bpp=0.0):
        """A Float64 form against the pipe that does its distance work: the FP32 pipe for the split form,
        the FP64 pipe for the exact form (the other fraction beside it)."""
        e = frac_entry(pairs, ms, F, p32 if split else p64, bpp)
        e["pipe"] = "fp32" if split else "fp64"
        other = roofline_pairs(F, p64 if split else p32, bpp, hbm)
        e["frac_of_fp64_roofline" if split else "frac_of_fp32_roofline"] = e["pairs_per_s"] / other
        return e

    if "cfg1" in which:
        log("cfg1")
        x, side = W.cfg1()
        xd = torch.from_numpy(x).to(dev)
        f = torch.zeros_like(xd)
        P = Plain(L, A, np.float64, 3, 1, stream)
        P.box(np.diag(side), A.CLM_ORTHO, 8.0)
        pairs = P.count([xd])
        R = candidates_per_hit(P.cell_size(), 8.0)
        res = {"workload": "uniform 100k f64 orthorhombic [0,100)^3 rc 8", "pairs": pairs, "candidates_per_hit": R}
        for opname in ("nl", "soft_energy", "soft_forces"):
            o = A.Outputs()
            o.forces_x = f.data_ptr()
            o.out_on_device = 1
            p = A.OpParams()
            for prec, tag in ((A.CLM_PREC_EXACT, "exact"), (A.CLM_PREC_SPLIT, "split")):
                L.clm_set_precision(P.h, prec)
                st_ms, k_ms, b_ms = P.timed([xd], A.OP[opname], p, o, steps, warmup, flush)
                F = 8 * R + F_OP[opname]
                e = form_entry(pairs, k_ms, F, tag == "split", 16.0 if opname == "nl" else 0.0)
                e.update({"step_ms": st_ms, "build_ms": b_ms, "step_pairs_per_s": pairs / (st_ms * 1e-3)})
                res[f"{opname}/{tag}"] = e
        P.close()
        out["cfg1"] = res

    if "cfg2_f64" in which:
        log("cfg2_f64")
        # the headline geometry with Float64 positions: the FP32-split form against the exact FP64 form
        x2, M2 = make_workload(64)
        xd = torch.from_numpy(x2.astype(np.float64)).to(dev)
        f = torch.zeros_like(xd)
        P = Plain(L, A, np.float64, 3, 1, stream)
        P.box(M2, A.CLM_TRICLINIC, CUTOFF)
        pairs = P.count([xd])
        R = candidates_per_hit(P.cell_size(), CUTOFF)
        p = A.OpParams()
        p.p[0], p.p[1], p.p[2], p.p[3] = 1.0, 1.0, 4.0, 4.0
        o = A.Outputs()
        o.forces_x = f.data_ptr()
        o.out_on_device = 1
        res = {"workload": "the headline fcc triclinic LJ workload with Float64 positions", "pairs": pairs,
               "candidates_per_hit": R}
        for prec, tag in ((A.CLM_PREC_EXACT, "exact"), (A.CLM_PREC_SPLIT, "split")):
            L.clm_set_precision(P.h, prec)
            st_ms, k_ms, b_ms = P.timed([xd], A.OP["lj_forces"], p, o, steps, warmup, flush)
            F = 8 * R + F_OP["lj_forces"]
            e = form_entry(pairs, k_ms, F, tag == "split")
            e.update({"step_ms": st_ms, "build_ms": b_ms})
            res[tag] = e
        res["split_over_exact"] = res["exact"]["kernel_ms"] / res["split"]["kernel_ms"]
        P.close()
        out["cfg2_f64"] = res

    if "cfg3" in which:
        log("cfg3")
        x, off, sides = W.cfg3()
        n = x.shape[0]
        xd = torch.from_numpy(x).to(dev)
        cells = np.repeat(sides[:, None], 3, axis=1)
        bs = pkg.BatchedSystems(positions=xd, offsets=off, unitcells=cells, cutoff=6.0)
        cnt = bs.run(pkg.Count())[0]
        pairs = int(cnt.sum())
        valid = bs.status() == 0
        h = sides / np.floor(sides / 6.0)
        Rs = np.array([candidates_per_hit([hh] * 3, 6.0) for hh in h])
        R = float(np.sum(Rs[valid] * cnt[valid]) / max(1, pairs))
        F = (8 * R + F_OP["nl"]) + (8 * R + F_OP["soft_energy"])  # one step: neighbour list + soft energy
        res = {"workload": "4096 uniform f64 systems, n log-uniform 64-20000, rho 0.1, rc 6 (NL + soft energy)",
               "n_particles": n, "pairs": pairs, "invalid_systems": int((~valid).sum()), "candidates_per_hit": R}
        tune = bs.autotune(pkg.NeighborList(), pkg.SoftEnergy(), reps=2)
        res["autotuned"] = tune
        for tag in ("exact", "split"):
            bs.set_precision(tag)
            bs.graph = True
            ts = []
            for k in range(warmup + steps):
                with torch.cuda.stream(stream):
                    flush.add_(1.0)
                torch.cuda.synchronize()
                bs.run(pkg.NeighborList(), pkg.SoftEnergy())
                if k >= warmup:
                    ts.append(bs.last_step()["step_ms"])
            ms = statistics.median(ts)
            e = form_entry(pairs, ms, F, tag == "split", 16.0)
            e.update({"graph_launches": bs.last_step()["launches"], "step_ms": ms})
            res[tag] = e
            bs.graph = False
        # the plain path on the same systems, one system at a time: the sum of its device time per system
        # (CUDA events around each build and map, the library's own timings), so that host overhead between
        # the systems is not counted against it
        P = Plain(L, A, np.float64, 3, 1, stream)
        o = A.Outputs()
        p = A.OpParams()
        dev_ms = {"exact": 0.0, "split": 0.0}
        for tag, prec in (("exact", A.CLM_PREC_EXACT), ("split", A.CLM_PREC_SPLIT)):
            L.clm_set_precision(P.h, prec)
            for s in range(len(sides)):
                if not valid[s]:
                    continue
                P.box(np.diag([sides[s]] * 3), A.CLM_ORTHO, 6.0)
                xs = xd[off[s]:off[s + 1]]
                for opname in ("nl", "soft_energy"):
                    P.step([xs], A.OP[opname], p, o)
                    bm, mm = C.c_float(), C.c_float()
                    L.clm_last_timings(P.h, C.byref(bm), C.byref(mm))
                    dev_ms[tag] += bm.value + mm.value
        P.close()
        res["plain_per_system"] = {t: {"device_ms": dev_ms[t], "pairs_per_s": pairs / (dev_ms[t] * 1e-3)}
                                   for t in dev_ms}
        res["batched_over_plain"] = {t: dev_ms[t] / res[t]["step_ms"] for t in ("exact", "split")}
        bs.close()
        del xd
        out["cfg3"] = res

    if "cfg4" in which:
        log("cfg4")
        x, Lb, t, eps, sig = W.cfg4()
        n = x.shape[0]
        xd = torch.from_numpy(x).to(dev)
        f = torch.zeros_like(xd)
        P = Plain(L, A, np.float32, 3, 1, stream)
        P.box(np.diag([Lb] * 3), A.CLM_ORTHO, 2.5)
        pairs = P.count([xd])
        R = candidates_per_hit(P.cell_size(), 2.5)
        ti = np.ascontiguousarray(t, np.int32)
        et, stb = np.ascontiguousarray(eps), np.ascontiguousarray(sig)
        p = A.OpParams()
        p.p[0], p.p[1], p.p[2], p.p[3] = 1.0, 1.0, 4.0, 4.0
        p.ntypes, p.types_x, p.eps_table, p.sig_table = 2, ti.ctypes.data, et.ctypes.data, stb.ctypes.data
        adj = np.zeros(32)
        o = A.Outputs()
        o.forces_x = f.data_ptr()
        o.out_on_device = 1
        o.adjoint = adj.ctypes.data
        res = {"workload": "200k f32 80:20 LJ mixture, jittered fcc rho 1.2, cubic, rc 2.5", "pairs": pairs,
               "candidates_per_hit": R}
        st_ms, k_ms, b_ms = P.timed([xd], A.OP["lj_adjoint"], p, o, steps, warmup, flush)
        e = frac_entry(pairs, k_ms, 8 * R + F_OP["lj_adjoint_types"], p32)
        e.update({"step_ms": st_ms, "build_ms": b_ms})
        res["adjoint"] = e
        st_ms, k_ms, b_ms = P.timed([xd], A.OP["lj_forces"], p, o, steps, warmup, flush)
        e = frac_entry(pairs, k_ms, 8 * R + F_OP["lj_forces_types"], p32)
        e.update({"step_ms": st_ms, "build_ms": b_ms})
        res["forces_only"] = e
        P.close()
        out["cfg4"] = res

    for dim, nset, key in ((3, 2_000_000, "cfg5"), (2, 2_000_000, "cfg5_2d"), (3, 200_000, "cfg5_small"),
                           (2, 200_000, "cfg5_2d_small")):
        if key not in which:
            continue
        log(key)
        x, y, vx, vy, side = W.cfg5(n=nset, dim=dim)
        bins = np.ascontiguousarray(W.cfg5_bins())
        xd, yd = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
        vxa, vya = np.ascontiguousarray(vx), np.ascontiguousarray(vy)
        P = Plain(L, A, np.float64, dim, 2, stream)
        P.box(np.diag(side), A.CLM_ORTHO, 25.0)
        p = A.OpParams()
        p.nbins, p.vel_x, p.vel_y, p.bins = 50, vxa.ctypes.data, vya.ctypes.data, bins.ctypes.data
        hc = np.zeros(50, np.int64)
        hs = np.zeros(50)
        o = A.Outputs()
        o.hist_count, o.hist_sum = hc.ctypes.data, hs.ctypes.data
        R = candidates_per_hit(P.cell_size()[:dim], 25.0, dim)
        res = {"workload": f"2 x {nset} f64 {dim}D uniform, side 250, rc 25, 50 log bins 0.1-25, v ~ N(0, 300^2)",
               "candidates_per_hit": R}
        pairs = None
        for prec, tag in ((A.CLM_PREC_SPLIT, "split"), (A.CLM_PREC_EXACT, "exact")):
            L.clm_set_precision(P.h, prec)
            st_ms, k_ms, b_ms = P.timed([xd, yd], A.OP["rhist"], p, o, 1 if key == "cfg5_2d" else max(1, steps // 5),
                                        1, flush)
            log(f"{key} {tag}: {k_ms:.1f} ms per map")
            if pairs is None:
                pairs = int(hc.sum())  # pairs with r >= 0.1 that fall in a bin
                res["pairs_in_bins"] = pairs
            e = form_entry(pairs, k_ms, 8 * R + F_OP["rhist"], tag == "split")
            e.update({"step_ms": st_ms, "build_ms": b_ms})
            res[tag] = e
        P.close()
        out[key] = res
    return out


def forms_summary(forms, build_roof):
    """Compact view of every measured form: name -> [pairs/s, fraction of its roofline, pipe]."""
    out = {}

    def add(name, e, pipe):
        if isinstance(e, dict) and "pairs_per_s" in e:
            out[name] = [float(f"{e['pairs_per_s']:.3g}"), float(f"{e.get('frac', float('nan')):.3g}"),
                         e.get("pipe", pipe)]

    for key, res in forms.items():
        if key in ("exact", "split"):
            out[f"headline/{key}"] = [float(f"{res['value']:.3g}"), None, "fp32"]
            continue
        if not isinstance(res, dict):
            continue
        for tag, e in res.items():
            add(f"{key}/{tag}", e, "fp32" if key == "cfg4" else "fp64")
        if "batched_over_plain" in res:
            out[f"{key}/batched_over_plain"] = {t: float(f"{v:.3g}") for t, v in res["batched_over_plain"].items()}
    if build_roof.get("frac") is not None:
        out["build/hbm"] = [float(f"{build_roof['achieved']:.3g}"), float(f"{build_roof['frac']:.3g}"), "hbm GB/s"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--ncell", type=int, default=64, help="fcc cells per side (64 -> 1,048,576 particles)")
    ap.add_argument("--cpu-steps", type=int, default=2, help="steps of the CPU baseline sample")
    ap.add_argument("--forms", default="cfg1,cfg2_f64,cfg3,cfg4,cfg5,cfg5_2d",
                    help="other configurations measured beside the headline (comma list, '' for none; "
                         "cfg5_small and cfg5_2d_small are 2 x 200k-point versions of the two-set histogram)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    threads = os.cpu_count() or 1

    x_host, M = make_workload(args.ncell)
    n = x_host.shape[0]

    if args.impl == "reference":
        if rank != 0:
            return 0
        pairs, dt = cpu_reference(x_host, M, args.steps, args.warmup, threads)
        v = pairs * args.steps / dt
        line = {"metric": METRIC, "value": v, "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference",
                "config": {"workload": WORKLOAD, "n_particles": n, "pairs_per_step": int(pairs), "cutoff": CUTOFF,
                           "cell": "triclinic", "op": "lj_energy_forces"},
                "cpu_baseline": {"value": v, "unit": "pairs/s", "cores": threads, "kind": "port",
                                 "sample": f"full workload, {args.steps} steps (OpenMP build and map on {threads} threads)"},
                "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__ as ge
    pkg = ge.load_package()
    pkg.build()
    L = pkg._abi.load()
    A = pkg._abi

    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    x_dev = torch.from_numpy(x_host).to(dev)
    f_dev = torch.zeros((n, 3), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)

    h = C.c_void_p()
    assert L.clm_create(A.CLM_F32, 3, 1, C.byref(h)) == 0
    assert L.clm_set_stream(h, C.c_void_p(stream.cuda_stream)) == 0
    Mf = np.ascontiguousarray(M.flatten(order="F"))
    assert L.clm_set_box(h, Mf.ctypes.data_as(C.POINTER(C.c_double)), A.CLM_TRICLINIC, CUTOFF, 1) == 0

    p = A.OpParams()
    p.p[0], p.p[1], p.p[2], p.p[3] = 1.0, 1.0, 4.0, 4.0
    o_dev = A.Outputs()
    o_dev.forces_x = f_dev.data_ptr()
    o_dev.out_on_device = 1

    def step_device():
        # new positions, then the map: clm_run rebuilds the updated cell list itself (as pairwise! after an
        # update of the positions does) and checks the build's totals with the map's results, one host
        # synchronization per step
        st = L.clm_set_positions(h, 0, C.c_void_p(x_dev.data_ptr()), n, 1)
        st = st or L.clm_run(h, A.OP["lj_forces"], C.byref(p), C.byref(o_dev))
        if st:
            buf = C.create_string_buffer(512)
            L.clm_last_error(h, buf, 512)
            raise RuntimeError(f"clm status {st}: {buf.value.decode()}")

    # pairs per step (untimed)
    L.clm_set_positions(h, 0, C.c_void_p(x_dev.data_ptr()), n, 1)
    oc = A.Outputs()
    assert L.clm_run(h, A.OP["count"], C.byref(A.OpParams()), C.byref(oc)) == 0
    pairs = int(oc.count)

    def timed(form):
        L.clm_set_precision(h, form)
        for _ in range(args.warmup):
            step_device()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        l0 = C.c_int64()
        L.clm_stats(h, C.byref(l0))
        tot_ms, kern_ms, bld_ms = 0.0, [], []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.add_(1.0)  # evict L2 between timed steps (outside the events)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step_device()
            e1.record(stream)
            e1.synchronize()
            tot_ms += e0.elapsed_time(e1)
            bm, mm = C.c_float(), C.c_float()
            L.clm_last_timings(h, C.byref(bm), C.byref(mm))
            kern_ms.append(mm.value)
            bld_ms.append(bm.value)
        torch.cuda.synchronize()
        timed.build_ms = statistics.median(bld_ms)
        l1 = C.c_int64()
        L.clm_stats(h, C.byref(l1))
        tot_ms = max_over_ranks(tot_ms, world, dev)
        return tot_ms, statistics.mean(kern_ms), (l1.value - l0.value)

    clocks = ClockSampler(local)
    clocks.start()
    t_exact, k_exact, launches = timed(A.CLM_PREC_EXACT)
    build_ms = timed.build_ms
    clk = clocks.stop()
    t_split, k_split, _ = timed(A.CLM_PREC_SPLIT)
    value = pairs * args.steps * world / (t_exact * 1e-3)
    split_value = pairs * args.steps * world / (t_split * 1e-3)

    # e2e: public C ABI with host buffers (pinned), copies inside the timed region
    L.clm_set_precision(h, A.CLM_PREC_EXACT)
    x_pin = torch.from_numpy(x_host).pin_memory()
    f_pin = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    o_host = A.Outputs()
    o_host.forces_x = f_pin.data_ptr()
    o_host.out_on_device = 0
    for _ in range(args.warmup):
        L.clm_set_positions(h, 0, C.c_void_p(x_pin.data_ptr()), n, 0)
        L.clm_run(h, A.OP["lj_forces"], C.byref(p), C.byref(o_host))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L.clm_set_positions(h, 0, C.c_void_p(x_pin.data_ptr()), n, 0)
        st = L.clm_run(h, A.OP["lj_forces"], C.byref(p), C.byref(o_host))
        assert st == 0
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    e2e = pairs * args.steps * world / t_e2e
    energy = o_host.scalar

    # roofline of the pair kernel (FP32 pipe): algorithmic flops per launch / kernel time
    box = np.zeros(3)
    cs = np.zeros(3)
    L.clm_get_box(h, None, cs.ctypes.data, None, None, None, None, None, None)
    fpp, R = flops_per_pair(cs, CUTOFF)
    peaks = C.CDLL(os.path.join(ge.PKG_DIR, "_build", "libclm_peaks.so"))
    peaks.clm_peak_fp32_gflops.restype = C.c_double
    peaks.clm_peak_fp32_gflops.argtypes = [C.c_int]
    fp32_peak = peaks.clm_peak_fp32_gflops(1 << 16) / 1e3  # TFLOP/s
    achieved = pairs * fpp / (k_exact * 1e-3) / 1e12
    # binning roofline (HBM): algorithmic bytes = 3s read + g (3s + 4) written per particle + ~12 B per cell
    info = [C.c_int64() for _ in range(4)]
    L.clm_get_celllist_info(h, 0, *[C.byref(v) for v in info])
    ncs = np.zeros(3, np.int64)
    L.clm_get_box(h, ncs.ctypes.data, None, None, None, None, None, None, None)
    copies, ncells = info[1].value, int(np.prod(ncs))
    build_bytes = n * 3 * 4 + copies * (3 * 4 + 4) + 12 * ncells
    hbm_peak = None
    mpj = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(mpj):
        hbm_peak = json.load(open(mpj)).get("hbm_gbs")
    build_gbs = build_bytes / (build_ms * 1e-3) / 1e9 if build_ms > 0 else None
    build_roof = {"bound": "hbm", "achieved": build_gbs, "peak": hbm_peak, "unit": "GB/s",
                  "frac": (build_gbs / hbm_peak) if (build_gbs and hbm_peak) else None,
                  "bytes_per_build": build_bytes, "copies": copies, "cells": ncells, "build_ms": build_ms,
                  "note": "cell-list build (wrap and images, cell scan, scatter, in-cell rank and gather) as a whole; latency-bound at this size"}
    # dram__bytes_read.sum + dram__bytes_write.sum of one launch of this kernel on this workload, from one
    # ncu capture recorded beside its summary in profiles/; a profiler cannot run inside the timed region,
    # so the figure is read from that record rather than measured here
    traffic = None
    if os.path.exists(TRAFFIC_RECORD):
        rec = json.load(open(TRAFFIC_RECORD))
        traffic = int(rec["dram_bytes_read"]) + int(rec["dram_bytes_write"])

    peaks.clm_peak_fp64_gflops.restype = C.c_double
    peaks.clm_peak_fp64_gflops.argtypes = [C.c_int]
    fp64_peak = peaks.clm_peak_fp64_gflops(1 << 12) / 1e3
    hbm = None
    mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(mp):
        hbm = json.load(open(mp)).get("hbm_gbs")
    forms_other = {}
    which = [w for w in args.forms.split(",") if w]
    if which:
        forms_other = measure_forms(pkg, L, A, dev, stream, flush,
                                    {"fp32_tflops": fp32_peak, "fp64_tflops": fp64_peak, "hbm_gbs": hbm or 6795.1},
                                    which, max(3, min(args.steps, 10)), 3)

    cpu = None
    if rank == 0 and args.cpu_steps > 0:
        try:
            cpairs, cdt = cpu_reference(x_host, M, args.cpu_steps, 0, threads)
            cpu = {"value": cpairs * args.cpu_steps / cdt, "unit": "pairs/s", "cores": threads, "kind": "port",
                   "sample": f"full workload, {args.cpu_steps} step(s), OpenMP build and map on {threads} threads"}
        except Exception as ex:  # pragma: no cover
            cpu = {"value": None, "unit": "pairs/s", "cores": threads, "kind": "port", "sample": f"failed: {ex}"}

    forms = {"exact": {"value": value, "kernel_ms": k_exact},
             "split": {"value": split_value, "kernel_ms": k_split, "ms_per_step": t_split / args.steps},
             **forms_other}
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_exact / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fcc + Gaussian jitter)",
        "config": {"workload": WORKLOAD, "n_particles": n, "pairs_per_step": pairs, "cutoff": CUTOFF,
                   "cell": "triclinic", "op": "lj_energy_forces", "l2": "flushed between steps (256 MiB write)"},
        "parallelism": f"replicas x{world}", "energy": energy,
        "forms": forms,
        "peaks": {"fp32_tflops": fp32_peak, "fp64_tflops": fp64_peak, "hbm_gbs": hbm,
                  "source": "FMA-loop probes (libclm_peaks.so) in this run; HBM from MEASURED_PEAKS.json"},
        "build_roofline": build_roof,
        "e2e": {"value": e2e, "unit": "pairs/s", "h2d_bytes_per_step": int(x_pin.numel() * 4),
                "d2h_bytes_per_step": int(f_pin.numel() * 4 + 8)},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak if fp32_peak > 0 else None, "traffic": traffic,
                     "kernel": "k_pairs<float,3,FORCES,exact>", "flops_per_pair": fpp, "candidates_per_hit": R,
                     "peak_source": "measured FP32 FMA throughput (libclm_peaks.so, same run)"},
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": launches,
        # last, so that it survives a tail of the output: every form's pairs/s, the fraction of its roofline
        # and the pipe it is measured against
        "forms_summary": forms_summary(forms, build_roof),
    }
    if rank == 0:
        print(json.dumps(line))
    L.clm_destroy(h)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

#!/usr/bin/env python
"""One q-point of the production-size RPA workload per step.

Workload (default ``--config grid120``): 120x120 k-grid (14400 FBZ points, Nsym=1),
30 bands (8 occupied), ~1500 plane-wave coefficients per band (igk-ordered
k+G spheres), NGloc = 91 local fields, nw = 1001 frequencies on 0-30 eV,
eta = 25 meV, q one grid step along Gamma-M.  A step computes, for that q:
the current-current correlation S0 and chi0 for pol xx and pol zz (Optabs:
vertices, S0 over -no..no, Qeff, KK) and the loss chain (Sloss: vertices,
S0, KK, eps = 1 - chi0 V, gjel, W).  Metric: q-point spectra per second.
With N ranks, rank r computes its own q-point (r + 1 grid steps) and the
step time is the slowest rank's (weak scaling, no collective on the data
path).

value : inputs resident in HBM (basis loaded once), outputs left on the device.
e2e   : the same step through the C ABI with host buffers: the basis is copied
        from page-locked host memory every step and S0 (xx, zz), Qeff, chi0
        (xx, zz, loss), W and eps^-1_00 are read back.
--impl reference : the CPU restatement of the reference (oracle/, OpenMP on
        all host cores) on a bounded k / frequency sample, extrapolated.
"""
from __future__ import annotations

import argparse
import importlib
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "2dmaterialsopticalprops_gb300"


ACC_DRAM_BYTES_PER_PAIR = 43.0e9 / 54.6e6
# DRAM bytes per FBZ k-point of the vertex launches (k_vertex_mn): ncu measured
# 16.0 + 0.55 GB (current, xx), 34.47 + 1.20 GB (current, xx and zz in one pass)
# and 1.31 + 0.18 GB (charge) for the 1600 k-points of the 40x40 case
VTX_DRAM_BYTES_PER_K_CURRENT = 16.56e9 / 1600
VTX_DRAM_BYTES_PER_K_PAIR = 35.67e9 / 1600
VTX_DRAM_BYTES_PER_K_CHARGE = 1.48e9 / 1600


def pkg(name):
    return importlib.import_module(f"{PKG}.{name}")


def config_of(name: str, q_steps: int):
    synth = pkg("synth")
    if name == "grid120":
        return synth.config_grid120(q_steps=q_steps)
    if name == "grid60":  # the grid120 workload on a 60x60 k-grid (profiling-size case)
        return synth.config_grid120(nk=60, q_steps=q_steps)
    if name == "grid40":  # the grid120 workload on a 40x40 k-grid (1.2 GB basis: ncu-capture size)
        return synth.config_grid120(nk=40, q_steps=q_steps)
    if name == "grid24":
        return synth.config_grid24()
    if name == "small":
        return synth.config_small(q_steps=q_steps)
    if name == "dyson301":  # a small k-grid with the large-W Dyson size: NGloc 301, nw 701 (profiling case)
        return synth.config_small(nk=8, nbnd=16, nocc=6, npw=600, nlf=301, lf="xyz", no=701, omax_ev=50.0,
                                  eta_ev=0.05, q_steps=q_steps)
    raise SystemExit(f"unknown config {name}")


def q_steps_of_rank(rank: int) -> int:
    """q-point of a rank: rank r computes q = (r + 1) grid steps along Gamma-M
    (independent q-points, weak scaling, no collective on the data path)."""
    return 1 + rank


def max_over_ranks(dist, value: float, device: str = "cuda") -> float:
    """The largest value over all ranks (the slowest rank's time); value
    itself without a process group."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_desc(s, name):
    c = s.cfg
    return {"workload": f"{name}: {c.nk}x{c.nk} k-grid, {c.nbnd} bands ({c.nocc} occ), ~{c.npw} coefficients, "
                        f"NGloc={s.nlf}, nw={s.no}, eta={c.eta_ev * 1000:.0f} meV; per q: Optabs xx+zz (S0, Qeff, "
                        f"KK) + Sloss (S0, KK, Dyson, W)",
            "ntot": int(s.ntot), "nbnd": int(s.nbnd), "npw_max": int(s.npwx), "ng": int(s.G.shape[0]),
            "nlf": int(s.nlf), "nw": int(s.no), "q_per_step": 1, "basis_gb": round(s.coeff.nbytes / 1e9, 2)}


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]), f[5:9]))
            except ValueError:
                pass
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [r for r in rows if r[2] > 200.0] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in load for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in load])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "power_w_max": max(r[2] for r in rows)}


# ---------------------------------------------------------------------------
# Optabs xx computes the zz vertices in the same pass (rpa_chi0_prefetch);
# --no-prefetch runs the two polarisations' vertex passes separately
PREFETCH = True


def run_step(ctx, s, rpa, host=None):
    """One q-point: Optabs xx, Optabs zz, Sloss + Dyson.  host: None (outputs
    stay on the device), {} (new host arrays) or the dict alloc_outputs()
    returns (caller-owned buffers, reused from step to step, as a driver
    reuses its S0 / chi0 / WT arrays)."""
    want = host is not None
    bufs = host if host else None
    out = {}
    for pol in ("xx", "zz"):
        if pol == "xx" and PREFETCH:
            ctx.chi0_prefetch("zz")
        b = bufs[pol] if bufs else None
        S0, Q = ctx.chi0(rpa.MODE_CURRENT, want=want, out=b[:2] if b else None, **rpa.optabs_args(s, pol))
        chi = ctx.kk(rpa.KK_OPTABS_COMPLEX, want=want, out=b[2] if b else None)
        out[pol] = (S0, Q, chi)
    b = bufs["loss"] if bufs else None
    S0, _ = ctx.chi0(rpa.MODE_CHARGE, want=want, out=(b[0], None) if b else None, **rpa.sloss_args(s))
    chi = ctx.kk(rpa.KK_SLOSS_REAL, want=want, out=b[1] if b else None)
    WT, _, head = ctx.dyson(s.c0, s.cfg.eps, want_wt=want, want_epsinv=False, want_head=want,
                            out=(b[2], None, b[3]) if b else None)
    out["loss"] = (S0, chi, WT, head)
    return out


def alloc_outputs(s, pinned: bool = True):
    """Host output buffers of one step (page-locked when pinned)."""
    import torch

    def buf(shape, dt):
        tdt = {np.complex128: torch.complex128, np.float64: torch.float64}[dt]
        if pinned:
            return torch.empty(shape, dtype=tdt, pin_memory=True).numpy()
        return np.empty(shape, dtype=dt)
    n, no = s.nlf, s.no
    cur = lambda: (buf((n, n, 2 * no + 1), np.complex128), buf((n, n), np.complex128),  # noqa: E731
                   buf((n, n, no - 1), np.complex128))
    return {"xx": cur(), "zz": cur(),
            "loss": (buf((n, n, no), np.float64), buf((n, n, no - 1), np.complex128),
                     buf((n, n, no - 1), np.complex128), buf((no - 1,), np.complex128))}


def step_work(ctx, s, rpa):
    """Algorithmic work of one step, from the library's own counters."""
    work = {}
    tot_acc = tot_vert = vbytes = 0.0
    # coefficients per FBZ k-point on the summed side (npw of K1; the legacy basis: ngd)
    nsum_k = float(np.sum(s.npw[np.asarray(s.K1) - 1])) if s.igk is not None else float(s.ngd) * s.ntot

    def vertex_bytes(st, nb):
        # algorithmic bytes of one vertex pass: the coefficients of the bands
        # read on both k-points (8 B per complex: fp16 hi/lo re/im), the int16
        # Gfast map, the FP32 complex vertex rows written
        return nb * 8.0 * nsum_k + 2.0 * s.nlf * nsum_k + 8.0 * s.nlf * st["transitions"]
    t = {"accumulate": 0.0, "vertices": 0.0, "pairs": 0.0, "kk": 0.0, "dyson": 0.0}
    n2 = float(s.nlf) ** 2
    for pol in ("xx", "zz"):
        if pol == "xx" and PREFETCH:
            ctx.chi0_prefetch("zz")
        ctx.chi0(rpa.MODE_CURRENT, want=False, **rpa.optabs_args(s, pol))
        st, tm = ctx.chi0_stats(), ctx.stage_times()
        tot_acc += 8.0 * n2 * st["sum_nwin"]
        tot_vert += 8.0 * st["vertex_macs"]
        if not PREFETCH:
            vbytes += vertex_bytes(st, 2 * s.nbnd)
        elif pol == "xx":
            # one pass for both polarisations: the coefficients and the map read
            # once, two sets of vertex rows written
            vbytes += vertex_bytes(st, 2 * s.nbnd) + 8.0 * s.nlf * st["transitions"]
        for k in ("accumulate", "vertices", "pairs"):
            t[k] += tm[k]
        ctx.kk(rpa.KK_OPTABS_COMPLEX, want=False)
        t["kk"] += ctx.stage_times()["kk"]
        work[pol] = st
    ctx.chi0(rpa.MODE_CHARGE, want=False, **rpa.sloss_args(s))
    st, tm = ctx.chi0_stats(), ctx.stage_times()
    tot_acc += 8.0 * n2 * st["sum_nwin"]
    tot_vert += 8.0 * st["vertex_macs"]
    vbytes += vertex_bytes(st, s.nbnd)
    for k in ("accumulate", "vertices", "pairs"):
        t[k] += tm[k]
    ctx.kk(rpa.KK_SLOSS_REAL, want=False)
    t["kk"] += ctx.stage_times()["kk"]
    ctx.dyson(s.c0, s.cfg.eps, want_wt=False, want_epsinv=False, want_head=False)
    t["dyson"] += ctx.stage_times()["dyson"]
    work["loss"] = st
    return {"acc_flops": tot_acc, "vertex_flops": tot_vert, "vertex_bytes": vbytes, "stage_ms": t, "stats": work}


class CpuSampler:
    """The CPU restatement (oracle, all host threads) timed on samples of one
    q-point of a workload and extrapolated to the whole q-point.

    The basis is built once, holding the coefficient blocks of every k-point
    that a sample of the run can draw; sample i times nk FBZ k-points evenly
    spaced over the grid with an offset that moves from sample to sample (so
    successive samples cover different k-points) for each of S0 xx / zz /
    loss (scaled by Ntot / nk), the KK transforms on an nb x nb block of the
    (G, G') pairs (scaled by NGloc^2 / nb^2) and the Dyson solve with the
    reference's 4-deep W loop on nthreads frequencies (scaled by nw / nws)."""

    def __init__(self, cfg_name: str, q_steps: int, nk: int | None = None, nsamples: int = 1,
                 full: bool = False):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        self.O = O
        synth = pkg("synth")
        cfg = config_of(cfg_name, q_steps)
        self.ntot = cfg.nk * cfg.nk
        self.nthreads = os.cpu_count() or 1
        self.full = full
        self.nk = self.ntot if full else min(self.ntot, nk or 2 * self.nthreads)
        self.stride = max(1, self.ntot // self.nk)
        ks = np.unique(np.concatenate([self.klist(i) for i in range(nsamples)]))
        self.s = synth.build(cfg, coeff_only=None if full else ks)

    def klist(self, i: int) -> np.ndarray:
        if self.full:
            return np.arange(self.ntot)
        return np.sort((np.arange(self.nk) * self.stride + 7 * i) % self.ntot)

    def run(self, i: int = 0):
        """(extrapolated seconds per q-point, parts, sample text, threads, wall seconds of the sample)."""
        O, s, nthreads = self.O, self.s, self.nthreads
        ks = self.klist(i)
        parts = {}
        w0 = time.perf_counter()
        for name, pol in (("optabs_xx", "xx"), ("optabs_zz", "zz"), ("sloss", None)):
            b = O.Bound(s, nthreads=nthreads, klist=ks, pol=pol or "xx")
            t0 = time.perf_counter()
            if pol:
                O.optabs_s0(b)
            else:
                O.sloss_s0(b)
            parts[name] = (time.perf_counter() - t0) / ks.size * self.ntot
        nb = s.nlf if self.full else min(8, s.nlf)
        So = np.random.default_rng(0).standard_normal((nb, nb, 2 * s.no + 1)) * (1 + 0j)
        t0 = time.perf_counter()
        O.kk_optabs(So, s.domega)
        parts["kk_optabs_x2"] = 2 * (time.perf_counter() - t0) * (s.nlf ** 2) / (nb * nb)
        Sl = np.random.default_rng(1).standard_normal((nb, nb, s.no))
        t0 = time.perf_counter()
        O.kk_sloss(Sl, s.domega)
        parts["kk_sloss"] = (time.perf_counter() - t0) * (s.nlf ** 2) / (nb * nb)
        nws = s.no - 1 if self.full else min(s.no - 1, nthreads)
        chi = np.random.default_rng(2).standard_normal((s.nlf, s.nlf, nws)) * 1e-3 + 0j
        V = O.genV(s)
        t0 = time.perf_counter()
        O.dyson(np.ascontiguousarray(chi), V, fast_wt=False, nthreads=nthreads)
        parts["dyson"] = (time.perf_counter() - t0) * (s.no - 1) / nws
        wall = time.perf_counter() - w0
        total = sum(parts.values())
        sample = (f"{ks.size} of {self.ntot} FBZ k-points for each of S0 xx/zz/loss (scaled by Ntot; offset "
                  f"moves per sample), KK on {nb}x{nb} of {s.nlf}x{s.nlf} (G,G') pairs, Dyson (4-deep WT loop) "
                  f"on {nws} of {s.no - 1} frequencies; extrapolated linearly")
        return total, parts, sample, nthreads, wall


def cpu_sample(cfg_name: str, q_steps: int, budget_s: float = 0.0):
    """One sample of CpuSampler: (extrapolated s per q, parts, sample, threads, system)."""
    cs = CpuSampler(cfg_name, q_steps, nk=4 * (os.cpu_count() or 1))
    total, parts, sample, nthreads, _ = cs.run(0)
    return total, parts, sample, nthreads, cs.s


def cpu_validate(cfg_name: str, nsamples: int = 3):
    """The sampled CPU estimate against a full run of the same q-point."""
    est = []
    cs = CpuSampler(cfg_name, 1, nsamples=nsamples)
    for i in range(nsamples):
        est.append(cs.run(i))
    del cs
    full = CpuSampler(cfg_name, 1, full=True)
    tf, pf, sf, thr, wall = full.run(0)
    te = float(np.mean([e[0] for e in est]))
    return {"config": cfg_name, "threads": thr, "full_s": tf, "full_parts_s": pf, "sampled_estimate_s": te,
            "sampled_estimates_s": [e[0] for e in est], "sample_wall_s": [e[4] for e in est],
            "estimate_error": te / tf - 1.0,
            "parts_error": {k: float(np.mean([e[1][k] for e in est]) / pf[k] - 1.0) for k in pf},
            "sample": est[0][2]}


# ---------------------------------------------------------------------------
# request mixes of the serving measurement: basis, q steps, NGloc, nw, local-field choice
SERVE_MIXES = {
    "grid60": dict(desc="grid60 basis resident (mixed path)", steps=(1, 16), nlf=(19, 92), no=(200, 1001), lf="z"),
    # MoS2-like resident basis: 72x72, 40 bands (13 occupied), ~2500 coefficients;
    # q ~ U(0.005, 0.5) 2pi/a as 1-31 grid steps along Gamma-M, NGloc 19-301, nw 200-2000
    "c4": dict(desc="72x72 basis, 40 bands (13 occ), ~2500 coefficients resident (mixed path)", steps=(1, 32),
               nlf=(19, 302), no=(200, 2001), lf="xyz"),
}


def serving_run(n_req: int = 32, rate: float = 200.0, nslots: int = 4, mem_gb: float = 40.0, seed: int = 5,
                mix: str = "grid60", batch_q: int = 0):
    """Request loop on a resident basis (mixed path): seeded Poisson arrivals of
    W (loss-function) and chi0 (Optabs xx) requests with the q, NGloc and nw
    ranges of SERVE_MIXES[mix], served by nslots shared contexts with
    continuous batching.  Latency = submission to completion (server clock)."""
    import threading
    rpa, synth = pkg("rpa"), pkg("synth")
    M = SERVE_MIXES[mix]
    if mix == "c4":
        s = synth.build(synth.config_grid120(nk=72, nbnd=40, nocc=13, npw=2500, nlf=19, no=1001, q_steps=1))
    else:
        s = synth.build(config_of("grid60", 1))
    parent = rpa.Context(precision=rpa.PREC_MIXED)
    parent.load_system(s)
    rng = np.random.default_rng(seed)

    def make(i):
        steps = int(rng.integers(*M["steps"]))
        km = synth.q_kmap(s, steps)
        nlf = int(rng.integers(*M["nlf"]))
        ilf, par = synth.local_fields(s, km["q"], 1e9, lf=M["lf"], nmax=nlf)
        no = int(rng.integers(*M["no"]))
        domega = s.domega * (s.no - 1) / (no - 1)
        if i % 2 == 0:
            args = dict(no=no, domega=domega, eta=s.eta, Vcell=s.Vcell, Gcar=s.Gcar, nocc=s.nocc)
            return dict(kind=rpa.REQ_W, kmap=km, ilf=ilf, parG=par, args=args, mode=rpa.MODE_CHARGE,
                        kk_variant=rpa.KK_SLOSS_REAL, c0=s.c0, eps=s.cfg.eps, want_chi0=False), (ilf.size, no, "W")
        a = rpa.optabs_args(s, "xx")
        a.update(no=no, domega=domega)
        return dict(kind=rpa.REQ_CHI0, kmap=km, ilf=ilf, parG=par, args=a, mode=rpa.MODE_CURRENT,
                    kk_variant=rpa.KK_OPTABS_COMPLEX), (ilf.size, no, "chi")

    reqs = [make(i) for i in range(n_req + 4)]
    srv = rpa.Server(parent, nslots=nslots, mem_bytes=mem_gb * 1e9, batch_q=batch_q)
    # warm-up: one request per slot at once, so that every slot's device
    # buffers reach their sizes before the timed stream
    for i in [srv.submit(**r) for r, _ in reqs[:4]]:
        srv.wait(i)
    reqs = reqs[4:]
    gaps = rng.exponential(1.0 / rate, size=n_req)
    ids = [None] * n_req
    t0 = time.perf_counter()

    def feeder():
        t = t0
        for i, ((r, _), g) in enumerate(zip(reqs, gaps)):
            t += g
            d = t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            ids[i] = srv.submit(**r)

    th = threading.Thread(target=feeder)
    th.start()
    th.join()
    res = [srv.wait(i)[1] for i in ids]
    t_end = time.perf_counter()
    n_batched = srv.batched_count()
    srv.close()
    parent.close()
    lat = np.array([r[0] for r in res])
    queue = np.array([r[1] for r in res])
    serv = np.array([r[2] for r in res])
    return {"workload": f"{M['desc']}; {n_req} requests, Poisson arrivals at {rate:g}/s "
                        f"(seed {seed}): W (loss) and chi0 (Optabs xx) alternating, q {M['steps'][0]}-"
                        f"{M['steps'][1] - 1} grid steps along Gamma-M, NGloc {M['nlf'][0]}-{M['nlf'][1] - 1}, "
                        f"nw {M['no'][0]}-{M['no'][1] - 1}; {nslots} slots, {mem_gb:g} GB admission budget",
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_queue_s": float(queue.mean()), "mean_service_s": float(serv.mean()),
            "batching_worker": {"batch_q": batch_q, "requests_batched": n_batched} if batch_q else None,
            "throughput_req_s": n_req / (t_end - t0), "n_requests": n_req, "slots": nslots,
            "ngloc_range": [int(min(r[1][0] for r in reqs)), int(max(r[1][0] for r in reqs))],
            "nw_range": [int(min(r[1][1] for r in reqs)), int(max(r[1][1] for r in reqs))]}


def dispersion_path(nk: int, n_q: int):
    """n_q commensurate q-points along Gamma-M-K of the nk x nk grid, as
    (steps along b1, steps along b2): Gamma-M is (s, 0), s = 1..nk/2, M-K is
    (nk/2 - j, 2j), j = 1..nk/6; n_q of them evenly spaced along the path."""
    pts = [(s_, 0) for s_ in range(1, nk // 2 + 1)] + [(nk // 2 - j, 2 * j) for j in range(1, nk // 6 + 1)]
    idx = np.unique(np.round(np.linspace(0, len(pts) - 1, n_q)).astype(int))
    return [pts[i] for i in idx]


def dispersion_run(parent, s, n_q: int = 64, nslots: int = 4, n_fp64: int = 8, no: int = 701,
                   eta_ev: float = 0.05, floor: float = 1e-3):
    """64-q loss-function dispersion (W and Im eps^-1 per q) on the resident
    grid120 basis: NGloc rising from 31 to 151 along the path, nw = 701 on
    0-30 eV, eta = 50 meV.  All q-points are submitted at once to a server of
    shared mixed-path contexts; a sample of q-points also runs on the plain
    FP64 GPU path for the speed ratio and the Im eps^-1 errors."""
    rpa, synth = pkg("rpa"), pkg("synth")
    own = parent is None
    if own:
        parent = rpa.Context(precision=rpa.PREC_MIXED)
        parent.load_system(s)
    path = dispersion_path(s.cfg.nk, n_q)
    n_q = len(path)
    # the q-points of the FP64 comparison: n_fp64 evenly spaced along the path
    # (0, 9, 18, ..., 63 for 64 q-points)
    fp64_sample = tuple(sorted({int(round(x)) for x in np.linspace(0, n_q - 1, n_fp64)}))
    domega = s.domega * (s.no - 1) / (no - 1)
    eta = eta_ev / 27.211386245988
    reqs, info = [], []
    for i, (a, b) in enumerate(path):
        km = synth.q_kmap(s, a, b)
        nlf = 31 + int(round(120 * i / max(n_q - 1, 1)))
        ilf, par = synth.local_fields(s, km["q"], 1e9, lf="xyz", nmax=nlf)
        args = dict(no=no, domega=domega, eta=eta, Vcell=s.Vcell, Gcar=s.Gcar, nocc=s.nocc)
        reqs.append(dict(kind=rpa.REQ_W, kmap=km, ilf=ilf, parG=par, args=args, mode=rpa.MODE_CHARGE,
                         kk_variant=rpa.KK_SLOSS_REAL, c0=s.c0, eps=s.cfg.eps))
        info.append((float(np.linalg.norm(km["q"])), int(ilf.size)))
    srv = rpa.Server(parent, nslots=nslots, mem_bytes=80e9)
    srv.wait(srv.submit(**reqs[-1]))  # warm-up at the largest NGloc
    t0 = time.perf_counter()
    ids = [srv.submit(**r) for r in reqs]
    res = [srv.wait(i) for i in ids]
    t_mixed = time.perf_counter() - t0
    srv.close()
    # the same 64 requests through rpa_batch: per-request setup, then per batch
    # one CUDA graph (grouped-tile S0 launches + KK + Dyson of every request);
    # once with one batch of 16 at a time, once with two batches of 8 that
    # alternate, the per-request part of one overlapping the other's graph
    breqs = [dict(kmap=r["kmap"], ilf=r["ilf"], parG=r["parG"], args=r["args"], c0=r["c0"], eps=r["eps"])
             for r in reqs]
    server_heads = [x[0]["head"] for x in res]

    def batched_run(bq, nobj):
        objs = [rpa.Batch(parent, max_q=bq) for _ in range(nobj)]
        for o in objs:
            o.run(breqs[-bq:])  # warm-up: buffers reach the largest NGloc's sizes
        chunks = [breqs[i:i + bq] for i in range(0, len(breqs), bq)]
        out, info = [], []
        t = time.perf_counter()
        pending = []  # objects with a launched batch, in launch order
        for j, ch in enumerate(chunks):
            o = objs[j % nobj]
            if o in pending:  # its previous batch (j - nobj) is the oldest pending one
                out += pending.pop(0).wait()
                info.append(o.info())
            o.launch(ch)
            pending.append(o)
        while pending:
            o = pending.pop(0)
            out += o.wait()
            info.append(o.info())
        dt = time.perf_counter() - t
        for o in objs:
            o.close()
        if any(st != 0 for st, _ in out):
            raise RuntimeError("batch failed")
        diff = max(float(np.abs(o["head"] - h).max() / np.abs(h).max()) for (_, o), h in zip(out, server_heads))
        return {"value": n_q / dt, "unit": "q-spectra/s", "s": dt, "batch_q": bq, "batches_alternating": nobj,
                "per_batch": [{k: (round(v, 4) if isinstance(v, float) else v) for k, v in x.items()} for x in info],
                "max_rel_diff_head_vs_server": diff}

    batched = batched_run(16, 1)
    batched["alternating_2x8"] = {k: v for k, v in batched_run(8, 2).items() if k != "per_batch"}
    batched["note"] = ("per-request setup (pairs, sort, vertices, B split) then one graph launch per batch of 16: "
                       "grouped-tile S0 launches per tile shape, S0 -> FP64, KK and Dyson of every request; "
                       "alternating_2x8: two batches of 8, the setup of one overlapping the other's graph")
    # FP64 GPU sample: the same requests, one at a time on an FP64 shared context
    c64 = rpa.shared_context(parent, rpa.PREC_FP64)
    t64, tmix_one, errs, stages = 0.0, 0.0, [], []
    cm = rpa.shared_context(parent)
    for qi in fp64_sample:
        r = reqs[qi]
        outs = []
        for c in (cm, c64):
            km = r["kmap"]
            t = time.perf_counter()
            c.kmap(km["ktot"], km["K1"], km["R1"], km["K2"], km["R2"], km["iG0"])
            c.set_q(km["q"], r["ilf"], r["parG"])
            c.chi0(rpa.MODE_CHARGE, want=False, **r["args"])
            c.kk(rpa.KK_SLOSS_REAL, want=False)
            _, _, head = c.dyson(r["c0"], r["eps"], want_wt=False)
            dt = time.perf_counter() - t
            if c is c64:
                t64 += dt
            else:
                tmix_one += dt
            outs.append(head)
            stages.append({"wall_ms": round(1e3 * dt, 2),
                           **{k: round(v, 2) for k, v in c.stage_times().items()},
                           **({"accum_tile": list(c.accum_tile())} if c is cm else {})})
        e = pkg("rpa").errstats(outs[0].imag, outs[1].imag, floor=floor)
        errs.append({"q_index": qi, "q_2pi_over_a": info[qi][0], "ngloc": info[qi][1],
                     "Im_epsinv_00": e, "mixed_ms": stages[-2], "fp64_ms": stages[-1]})
    c64.close()
    cm.close()
    if own:
        parent.close()
    return {"workload": f"{n_q} q-points along Gamma-M-K (|q| {info[0][0]:.4f}-{info[-1][0]:.3f} 2pi/a) on the "
                        f"grid120 basis; loss chain per q (S0, KK, FP64 Dyson, W, Im eps^-1), NGloc 31-151 rising "
                        f"along the path, nw={no}, eta={eta_ev * 1000:.0f} meV; mixed path: rpa_batch, batches of "
                        f"16 q-points (one CUDA graph each); also all 64 submitted at once to {nslots} shared contexts",
            "n_q": n_q, "value": batched["value"], "unit": "q-spectra/s", "mixed_s": batched["s"],
            "path": "rpa_batch: batches of 16 q-points, one CUDA graph each (graph_batched)",
            "graph_batched": batched,
            "server_concurrent": {"value": n_q / t_mixed, "s": t_mixed,
                                  "note": f"all 64 submitted at once to a server of {nslots} shared contexts"},
            "mean_service_s": float(np.mean([x[1][2] for x in res])),
            "fp64_sample": {"q_indices": list(fp64_sample), "ngloc": [info[i][1] for i in fp64_sample],
                            "fp64_s": t64, "mixed_s_one_at_a_time": tmix_one,
                            "fp64_q_spectra_s_est": len(fp64_sample) / t64,
                            "mixed_over_fp64_same_q": t64 / tmix_one,
                            "mixed_batched_over_fp64": batched["value"] / (len(fp64_sample) / t64),
                            "mixed_server_over_fp64": (n_q / t_mixed) / (len(fp64_sample) / t64),
                            "note": f"FP64 rate from {len(fp64_sample)} q-points evenly spaced along the path "
                                    f"(NGloc {info[fp64_sample[0]][1]}-{info[fp64_sample[-1]][1]}), run one at "
                                    f"a time; the mixed rate is the batched 64-q run"},
            "max_elem_rel_Im_epsinv_00": max(x["Im_epsinv_00"]["elem_max"] or 0.0 for x in errs),
            "error_floor": f"element-wise relative error over frequencies with |Im eps^-1_00| >= {floor:g} "
                           f"x its maximum; normwise = max|a-b| / max|b|; rms = ||a-b|| / ||b||",
            "errors_vs_fp64_gpu": errs}


def c5_config(nk: int):
    """Large screened interaction: MoS2-like cell stand-in (the synthetic
    hexagonal cell), 80 bands (13 occupied), ~4000 coefficients, NGloc = 301,
    nw = 701 on 0-50 eV, eta = 50 meV."""
    return pkg("synth").config_grid120(nk=nk, nbnd=80, nocc=13, npw=4000, nlf=301, lf="xyz", no=701,
                                       omax_ev=50.0, eta_ev=0.05)


def kmap_run(nk: int = 120, oracle_sample: int = 24):
    """The drivers' k-point bookkeeping for one q on a 120x120 hexagonal grid
    with the C6v point group (12 operations; 1261 IBZ points): genFBZ,
    findKinIBZ and findKQinBZ on the device (host-to-host wall time, 5 repeats,
    best), and the oracle's loop-for-loop restatement (pure Python) on a
    sample of FBZ points, scaled to the grid."""
    rpa, synth = pkg("rpa"), pkg("synth")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    a0, c0, V, KC = synth.hex_cell(2.46, 20.0)
    nsym, R, RI = synth.hex_symmetry()
    kI = synth.mp_ibz(KC, nk, R, nsym)
    miller, G = synth.g_list(KC, 3.5 ** 2)
    q = KC.T[0] / nk
    ctx = rpa.Context()
    ctx.set_gvectors(miller, G, KC)
    ctx.set_symmetry(nsym, R, RI)
    best = None
    for _ in range(5):
        t0 = time.perf_counter()
        ktot = ctx.gen_fbz(kI)
        t1 = time.perf_counter()
        ctx.find_k_ibz(ktot, kI)
        t2 = time.perf_counter()
        ctx.find_kq(ktot, kI, q)
        t3 = time.perf_counter()
        tt = (1e3 * (t1 - t0), 1e3 * (t2 - t1), 1e3 * (t3 - t2))
        best = tt if best is None or sum(tt) < sum(best) else best
    ctx.close()
    # CPU baseline: the oracle's findKQinBZ on a sample of FBZ points
    rng = np.random.default_rng(5)
    idx = np.sort(rng.choice(ktot.shape[0], size=oracle_sample, replace=False))
    t0 = time.perf_counter()
    orc.find_kq(ktot, kI, RI, nsym, G, q, 1e-4, points=idx)
    t_kq = (time.perf_counter() - t0) / oracle_sample * ktot.shape[0]
    return {"workload": f"{nk}x{nk} hexagonal grid, C6v (12 operations), {kI.shape[0]} IBZ points, "
                        f"{ktot.shape[0]} FBZ points, {G.shape[0]} G vectors, q one grid step along Gamma-M",
            "device_ms": {"gen_fbz": round(best[0], 2), "find_k_ibz": round(best[1], 2), "find_kq": round(best[2], 2)},
            "cpu_baseline": {"find_kq_s": round(t_kq, 1), "kind": "port", "cores": 1,
                             "sample": f"findKQinBZ restated loop for loop (pure Python) for {oracle_sample} of "
                                       f"{ktot.shape[0]} FBZ points, scaled by the point count"}}


def c5_run(n_q: int = 16, nk_full: int = 96, nk_check: int = 24, q_check=(1, 8), autotune: bool = True,
           floor: float = 1e-3):
    """W(q, w) for 16 q-points at full size on the mixed path (timed), and the
    mixed-vs-FP64 comparison (time ratio, per-q normwise / RMS / element-wise
    error of Im W and Im eps^-1_00) on the q-points q_check of the same
    workload on an nk_check x nk_check k-grid (nk_check = nk_full: the full
    size itself, on the same resident basis)."""
    rpa, synth = pkg("rpa"), pkg("synth")

    def w_chain(c, s, steps):
        km = synth.q_kmap(s, steps)
        c.kmap(km["ktot"], km["K1"], km["R1"], km["K2"], km["R2"], km["iG0"])
        c.set_q(km["q"], s.ilf, s.parG)
        c.chi0(rpa.MODE_CHARGE, want=False, **rpa.sloss_args(s))
        c.kk(rpa.KK_SLOSS_REAL, want=False)
        WT, _, head = c.dyson(s.c0, s.cfg.eps, want_wt=True)
        return WT, head

    def check(cm, s):
        c64 = rpa.shared_context(cm, rpa.PREC_FP64)
        errs, tm, t64 = [], 0.0, 0.0
        for st in q_check:
            t = time.perf_counter()
            Wm, hm = w_chain(cm, s, st)
            tm += time.perf_counter() - t
            t = time.perf_counter()
            W6, h6 = w_chain(c64, s, st)
            t64 += time.perf_counter() - t
            errs.append({"q_steps": st, "Im_W": rpa.errstats(Wm.imag, W6.imag, floor=floor),
                         "Im_W_00": rpa.errstats(Wm[0, 0].imag, W6[0, 0].imag, floor=floor),
                         "Im_epsinv_00": rpa.errstats(hm.imag, h6.imag, floor=floor)})
        c64.close()
        return {"grid": f"{s.cfg.nk}x{s.cfg.nk}", "mixed_s": tm, "fp64_s": t64, "mixed_over_fp64": t64 / tm,
                "errors_vs_fp64_gpu": errs,
                "error_floor": f"element-wise relative error where |b| >= {floor:g} max|b|"}

    chk = None
    if nk_check != nk_full:
        s = synth.build(c5_config(nk_check))
        cm = rpa.Context(precision=rpa.PREC_MIXED)
        cm.load_system(s)
        chk = check(cm, s)
        cm.close()
        del s
    # full size, mixed path
    t0 = time.perf_counter()
    s = synth.build(c5_config(nk_full))
    cm = rpa.Context(precision=rpa.PREC_MIXED)
    cm.load_system(s)
    t_setup = time.perf_counter() - t0
    steps = list(range(1, n_q + 1))
    w_chain(cm, s, steps[0])  # warm-up (buffers reach their sizes)
    vert_default = cm.stage_times()["vertices"]
    tune = None
    if autotune:
        # vertex tile autotuner on the first q-point; later q-points use its choice
        t = time.perf_counter()
        best = cm.autotune(rpa.MODE_CHARGE, **rpa.sloss_args(s))
        tune = {"tune_s": time.perf_counter() - t, "best_vertex_ms": best, "default_vertex_ms": vert_default,
                "table": json.loads(cm.tune_export())["vertex"]}
    t = time.perf_counter()
    for st in steps:
        w_chain(cm, s, st)
    t_full = time.perf_counter() - t
    st_times = cm.stage_times()
    if nk_check == nk_full:
        chk = check(cm, s)
    cm.close()
    return {"workload": f"large W: {nk_full}x{nk_full} k-grid, 80 bands (13 occ), ~4000 coefficients, "
                        f"NGloc=301, nw=701 on 0-50 eV, eta=50 meV, {n_q} q-points (1..{n_q} grid steps along "
                        f"Gamma-M); loss chain per q (S0, KK, FP64 Dyson, W)",
            "n_q": n_q, "mixed_s": t_full, "value": n_q / t_full, "unit": "q-spectra/s", "setup_s": t_setup,
            "last_q_stage_ms": st_times, "autotune": tune, "check": chk}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="grid120")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 GPU comparison step")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-validate", default=None, metavar="CONFIG",
                    help="time the CPU restatement on a full q-point of CONFIG and compare it with its sampled estimate")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-serve", action="store_true", help="skip the request-loop (serving) measurement")
    ap.add_argument("--c5", action="store_true",
                    help="also run the large-W workload (96x96, 80 bands, 4000 coefficients, NGloc 301; adds minutes)")
    ap.add_argument("--c5-check-nk", type=int, default=24,
                    help="k-grid of the C5 mixed-vs-FP64 check (96: the full size, two q-points, ~15 min)")
    ap.add_argument("--serve-c4", action="store_true",
                    help="also run the request loop on the MoS2-like 72x72 / 40-band / 2500-coefficient basis")
    ap.add_argument("--kmap", action="store_true",
                    help="also time the k-point bookkeeping (genFBZ / findKinIBZ / findKQinBZ) on a 120x120 C6v grid")
    ap.add_argument("--no-dispersion", action="store_true",
                    help="skip the 64-q loss-function dispersion (mixed path batched, FP64 GPU path on 8 q-points)")
    ap.add_argument("--dispersion", action="store_true",
                    help="run the dispersion on --config's basis too (it runs on grid120 by default)")
    ap.add_argument("--no-prefetch", action="store_true",
                    help="separate vertex passes for Optabs xx and zz (default: one pass, rpa_chi0_prefetch)")
    args = ap.parse_args()
    global PREFETCH
    PREFETCH = not args.no_prefetch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo" if args.impl == "reference" else "nccl")

    if args.cpu_validate:
        print(json.dumps(cpu_validate(args.cpu_validate)), flush=True)
        return

    if args.impl == "reference":
        if rank != 0:
            return
        cs = CpuSampler(args.config, 1, nsamples=args.warmup + args.steps)
        vals, walls = [], []
        for i in range(args.warmup + args.steps):
            tq, parts, sample, cores, wall = cs.run(i)
            if i >= args.warmup:
                vals.append(1.0 / tq)
                walls.append(wall)
        s = cs.s
        v = float(np.median(vals))
        cfgd = workload_desc(s, args.config)
        cfgd.update({"l2": "n/a (CPU; per-k working sets far below the host caches' size are not the bound)",
                     "parallelism": f"OpenMP over FBZ k-points, {cores} host threads",
                     "precision_path": "fp64 (oracle restatement of the reference loops)"})
        # a step is one bounded sample (a fraction of the q-point); value is the
        # extrapolated whole-q-point rate, ms_per_step the sample's wall time
        line = {"metric": "q-point chi/W spectra/sec", "value": v, "unit": "q-spectra/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.median(walls)),
                "q_fraction_per_step": float(np.median(walls)) * v, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "impl": "reference",
                "config": cfgd,
                "cpu_baseline": {"value": v, "unit": "q-spectra/s", "cores": cores, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": v, "unit": "q-spectra/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "parts_s": parts}
        print(json.dumps(line), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    rpa, synth = pkg("rpa"), pkg("synth")
    pkg("build").build()
    q_steps = q_steps_of_rank(rank)
    cfg = config_of(args.config, q_steps)
    t0 = time.time()
    s = synth.build(cfg)
    t_gen = time.time() - t0
    prec = rpa.PREC_MIXED if args.precision == "mixed" else rpa.PREC_FP64
    ctx = rpa.Context(device=local, precision=prec)
    ctx.load_system(s)
    stream = torch.cuda.ExternalStream(ctx.stream_handle())

    for _ in range(args.warmup):
        run_step(ctx, s, rpa)
    work = step_work(ctx, s, rpa)

    sampler = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    l0 = ctx.launch_count()
    ev0.record(stream)
    for _ in range(args.steps):
        run_step(ctx, s, rpa)
    ev1.record(stream)
    launches = ctx.launch_count() - l0
    torch.cuda.synchronize()
    ctx.synchronize()
    clocks = sampler.stop()
    ms = max_over_ranks(dist, ev0.elapsed_time(ev1) / args.steps)
    if dist:
        dist.barrier()
    value = world * 1000.0 / ms

    e2e = None
    out = None
    if not args.no_e2e:
        # the basis comes from page-locked host memory every step; the step's
        # spectra go to caller-owned page-locked buffers allocated once (as a
        # driver reuses its output arrays from q-point to q-point)
        pinned = torch.empty(s.coeff.shape, dtype=torch.complex128, pin_memory=True)
        pc = pinned.numpy()
        pc[...] = s.coeff
        bufs = alloc_outputs(s, pinned=True)
        h2d = pc.nbytes + s.E.nbytes + s.npw.nbytes + (s.igk.nbytes if s.igk is not None else 0) + \
            s.ktot.nbytes + 5 * s.K1.nbytes + s.q.nbytes + s.ilf.nbytes + s.parG.nbytes
        d2h = sum(a.nbytes for v in bufs.values() for a in v)
        e2e_ms, parts = [], {"load_basis": [], "kmap_set_q": [], "step": []}
        for i in range(1 + args.steps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            h0 = time.perf_counter()
            ctx.load_basis(s.npw, s.igk, pc, s.E)
            h1 = time.perf_counter()
            ctx.kmap(s.ktot, s.K1, s.R1, s.K2, s.R2, s.iG0)
            ctx.set_q(s.q, s.ilf, s.parG)
            h2 = time.perf_counter()
            out = run_step(ctx, s, rpa, host=bufs)
            h3 = time.perf_counter()
            e1.record(stream)
            torch.cuda.synchronize()
            if i > 0:
                e2e_ms.append(e0.elapsed_time(e1))
                for k, v in (("load_basis", h1 - h0), ("kmap_set_q", h2 - h1), ("step", h3 - h2)):
                    parts[k].append(1e3 * v)
        ems = max_over_ranks(dist, float(np.median(e2e_ms)))
        e2e = {"value": world * 1000.0 / ems, "unit": "q-spectra/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": ems,
               "parts_ms": {k: round(float(np.median(v)), 1) for k, v in parts.items()},
               "host_buffers": "inputs and outputs page-locked, outputs allocated once and reused"}
        # the same step once with fresh pageable output arrays (np.zeros per call,
        # first touch of every page during the read-back): for comparison only
        torch.cuda.synchronize()
        h0 = time.perf_counter()
        run_step(ctx, s, rpa, host={})
        e2e["pageable_fresh_outputs_step_ms"] = round(1e3 * (time.perf_counter() - h0), 1)

    # plain FP64 GPU path on the same inputs: its time per q-point and the
    # mixed path's errors against it (one step, host outputs)
    fp64 = None
    if args.precision == "mixed" and not args.no_fp64 and out is not None:
        mixed_out = {k: tuple(None if a is None else a.copy() for a in v) for k, v in out.items()}
        ctx.close()
        ctx64 = rpa.Context(device=local, precision=rpa.PREC_FP64)
        ctx64.load_system(s)
        st64 = torch.cuda.ExternalStream(ctx64.stream_handle())
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        f0.record(st64)
        ref = run_step(ctx64, s, rpa, host={})
        f1.record(st64)
        torch.cuda.synchronize()
        ms64 = f0.elapsed_time(f1)
        ctx64.close()

        err = rpa.errstats
        errs = {"S0_xx": err(mixed_out["xx"][0], ref["xx"][0]), "chi0_xx": err(mixed_out["xx"][2], ref["xx"][2]),
                "S0_zz": err(mixed_out["zz"][0], ref["zz"][0]), "chi0_zz": err(mixed_out["zz"][2], ref["zz"][2]),
                "S0_loss": err(mixed_out["loss"][0], ref["loss"][0]), "W": err(mixed_out["loss"][2], ref["loss"][2]),
                "Im_W": err(mixed_out["loss"][2].imag, ref["loss"][2].imag),
                "Im_epsinv_00": err(mixed_out["loss"][3].imag, ref["loss"][3].imag)}
        fp64 = {"ms_per_step": ms64, "value": 1000.0 / ms64, "unit": "q-spectra/s",
                "mixed_over_fp64": ms64 / ms, "errors_vs_fp64_gpu": errs}
        ctx = None

    # rooflines of the vertex and accumulation stages from the library's CUDA
    # events; `roofline` is the one with the larger share of the step
    sm = work["stage_ms"]
    acc_s = sm["accumulate"] / 1000.0
    vtx_s = sm["vertices"] / 1000.0
    achieved_tf = work["acc_flops"] / acc_s / 1e12 if acc_s > 0 else None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs")
    hbm_src = "MEASURED_PEAKS.json hbm_gbs" if hbm else "fallback 6800 GB/s (no MEASURED_PEAKS.json)"
    hbm = hbm or 6800.0
    vtx_gbs = work["vertex_bytes"] / vtx_s / 1e9 if vtx_s > 0 else None
    roof_vtx = {"bound": "hbm", "achieved": vtx_gbs, "peak": hbm, "unit": "GB/s",
                "frac": (vtx_gbs / hbm) if vtx_gbs else None, "peak_source": hbm_src,
                "bytes_per_step": work["vertex_bytes"],
                "byte_count": "sum over vertex passes of 8*Nb*sum_k NGd + 2*NG*sum_k NGd + 8*NG*T per row set "
                              "(Nb: bands read on both k-points; int16 Gfast map; FP32 rows out; the xx + zz "
                              "pass writes two row sets)",
                "vertex_tflops": (work["vertex_flops"] / vtx_s / 1e12) if vtx_s > 0 else None}
    if args.precision == "fp64":
        roof_vtx.update({"kernel": "k_vertex_fp64", "traffic": None})
        roof_acc = {"bound": "fp64", "achieved": achieved_tf, "peak": 1.25, "unit": "TFLOP/s",
                    "frac": (achieved_tf / 1.25) if achieved_tf else None, "traffic": None,
                    "peak_source": "nominal GB300 FP64 rate (no measured FP64 peak in MEASURED_PEAKS.json)",
                    "kernel": "k_accum_fp64 (+ per-chunk calls)",
                    "flops_per_step": work["acc_flops"], "flop_count": "8*NGloc^2*sum_t N_win(t)"}
    else:
        if PREFETCH:
            roof_vtx.update({"kernel": "k_vertex_mn (Optabs xx and zz: one current pass; Sloss: charge), "
                                       "2 launches per step",
                             "traffic": (VTX_DRAM_BYTES_PER_K_PAIR + VTX_DRAM_BYTES_PER_K_CHARGE) * s.ntot,
                             "traffic_basis": "DRAM bytes of the step's two vertex launches (xx + zz current; "
                                              "charge), per k-point from an ncu capture of the 40x40 case, times "
                                              "this workload's FBZ k-points (the passes bytes_per_step counts)"})
        else:
            roof_vtx.update({"kernel": "k_vertex_mn (Optabs xx, zz: current; Sloss: charge), 3 launches per step",
                             "traffic": (2 * VTX_DRAM_BYTES_PER_K_CURRENT + VTX_DRAM_BYTES_PER_K_CHARGE) * s.ntot,
                             "traffic_basis": "DRAM bytes of the step's three vertex launches (xx, zz current; "
                                              "charge), per k-point from an ncu capture of the 40x40 case, times "
                                              "this workload's FBZ k-points (the passes bytes_per_step counts)"})
        pk = peaks.get("bf16_tflops_sustained", 1700.0)
        # DRAM bytes of one complex (Optabs) accumulation launch: ncu measured
        # 39.9 + 3.1 GB for 54.6 M (transition, frequency) pairs on the 60x60
        # case (rows costliest first), scaled here by this workload's pairs
        # per launch
        nwin = [work["stats"][p]["sum_nwin"] for p in ("xx", "zz")]
        traffic = ACC_DRAM_BYTES_PER_PAIR * sum(nwin) / len(nwin)
        roof_acc = {"bound": "tensor", "achieved": achieved_tf, "peak": pk, "unit": "TFLOP/s",
                    "frac": (achieved_tf / pk) if achieved_tf else None, "traffic": traffic,
                    "kernel": "k_accum_ws (Optabs xx, zz: complex S0; Sloss: real S0), 3 launches per step",
                    "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (kernel timed inside a long step)",
                    "flops_per_step": work["acc_flops"], "flop_count": "8*NGloc^2*sum_t N_win(t)",
                    "traffic_basis": "GB per complex launch scaled from an ncu capture of the 60x60 case"}
    roof_vtx["stage_ms_per_step"] = sm["vertices"]
    roof_acc["stage_ms_per_step"] = sm["accumulate"]
    roof = dict(roof_vtx if sm["vertices"] >= sm["accumulate"] else roof_acc)
    roof["stage"] = "vertices" if sm["vertices"] >= sm["accumulate"] else "accumulate"
    roof_stages = {"vertices": roof_vtx, "accumulate": roof_acc}

    cpu = None
    if not args.no_cpu and rank == 0:
        tq, parts, sample, cores, _ = cpu_sample(args.config, q_steps, args.cpu_budget)
        cpu = {"value": 1.0 / tq, "unit": "q-spectra/s", "cores": cores, "kind": "port", "sample": sample,
               "parts_s": {k: round(v, 3) for k, v in parts.items()}}

    serving = disp = None
    if rank == 0 and not args.no_serve and args.precision == "mixed":
        serving = serving_run()
        serving["with_batching_worker"] = serving_run(batch_q=8)
    if rank == 0 and not args.no_dispersion and args.precision == "mixed" and (args.config == "grid120" or
                                                                              args.dispersion):
        disp = dispersion_run(ctx, s)
    kmap = kmap_run() if rank == 0 and args.kmap else None
    serving_c4 = None
    if rank == 0 and args.serve_c4 and args.precision == "mixed":
        serving_c4 = serving_run(mem_gb=120.0, mix="c4")
    c5 = None
    if rank == 0 and args.c5 and args.precision == "mixed":
        if ctx is not None:
            ctx.close()
            ctx = None
        c5 = c5_run(nk_check=args.c5_check_nk)

    if rank == 0:
        cfgd = workload_desc(s, args.config)
        cfgd.update({"l2": "inputs larger than L2 (basis %.1f GB resident)" % (s.coeff.nbytes / 1e9),
                     "parallelism": f"q-sharded x{world}" if world > 1 else "single GPU",
                     "precision_path": args.precision, "setup_s": round(t_gen, 1),
                     "vertex_passes": ("Optabs xx and zz share one vertex pass (rpa_chi0_prefetch)" if PREFETCH
                                       else "one vertex pass per polarisation")})
        line = {"metric": "q-point chi/W spectra/sec", "value": value, "unit": "q-spectra/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f16x3->f32 (vertices, S0), f32 (KK), f64 (Dyson)",
                "data": "synthetic (seeded QE-layout Bloch basis)", "config": cfgd, "clocks": clocks,
                "gpu_launches": launches, "roofline": roof, "roofline_stages": roof_stages,
                "cpu_baseline": cpu, "e2e": e2e,
                "stage_ms_per_step": {k: round(v, 3) for k, v in sm.items()},
                "fp64_gpu": fp64, "serving": serving, "dispersion": disp, "c5": c5, "kmap": kmap,
                "serving_c4": serving_c4}
        print(json.dumps(line), flush=True)
    if ctx is not None:
        ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""Benchmark of the DNS-aided LES hot path on one GB300 (or N replicas).

Workload (one "step"): one classical RK4 step of the 512^3 periodic
staggered-grid Navier-Stokes DNS (nu = 1/2000, FFT pressure projection at
each of the 4 stages) with the exact closure evaluated at every stage for a
64^3 (volume filter, ratio 8) and a 128^3 (volume filter, ratio 4) LES grid,
each LES advanced with and without the closure; seeded spectral initial
condition with k0 = 6 normalised to unit kinetic energy.  Metric:
cell-updates/s = 512^3 DNS cells x RK4 steps / second.

``--impl reference`` times the CPU restatement of the same path on the host
cores (the reference is Julia, which is not installed).
Multi-GPU runs are independent replicas (each rank its own solve; no
collective on the data path): ``value`` sums all ranks' cell updates over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "exactclosure.jl_gb300"))


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--precision", default="f64", choices=["f64", "f32"])
    ap.add_argument("--les", default="8:volume,4:volume")
    ap.add_argument("--kpeak", type=float, default=6.0)
    ap.add_argument("--visc", type=float, default=1 / 2000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-forms", action="store_true")
    ap.add_argument("--serve-only", action="store_true")
    ap.add_argument("--serve-steps", type=int, default=200, help="RK4 steps per solve of the serving stream")
    ap.add_argument("--no-fp64-stream", action="store_true")
    ap.add_argument("--no-burgers", action="store_true")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-c1", action="store_true")
    ap.add_argument("--only", default="", choices=["", "burgers", "large", "learned", "c1", "rhs"],
                    help="run one side workload alone and print its JSON object")
    ap.add_argument("--burgers-samples", type=int, default=1000)
    ap.add_argument("--burgers-tstop", type=float, default=0.1)
    ap.add_argument("--large-steps", type=int, default=300,
                    help="steps of the 1024^3 run (pairs every 10 steps; the learned closure trains on them)")
    ap.add_argument("--learned-steps", type=int, default=1000, help="Adam steps of the learned closure")
    ap.add_argument("--learned-les-steps", type=int, default=200,
                    help="steps of the learned-closure LES in lockstep with the 1024^3 DNS")
    ap.add_argument("--forms-steps", type=int, default=200,
                    help="steps of the FP32-vs-FP64 error comparison (0: skip)")
    return ap.parse_args()


def les_list(spec):
    out = []
    for item in spec.split(","):
        if item:
            r, k = item.split(":")
            out.append((int(r), k))
    return out


def measured_peaks() -> dict:
    """MEASURED_PEAKS.json, or the fallback figures (6.8 TB/s, 1.9 PFLOP/s bf16)."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        d["source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit())
        mx = max((float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(self.rows)}


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement on the host cores)
# ---------------------------------------------------------------------------
def cpu_sample(n_full: int, les, kpeak: float, visc: float, budget_s: float = 20.0):
    """Time the oracle's RK4 DNS-aided step on a bounded sample of the workload.

    Preference: the C/OpenMP restatement (oracle/cpu_ref) on the full grid,
    one RK4 stage per call; else the NumPy restatement on a smaller grid with
    the same filter ratios."""
    from oracle import cpu_ref

    if cpu_ref.available():
        r = cpu_ref.time_stages(n_full, les, kpeak, visc, budget_s)
        return {"value": r["cell_updates_per_s"], "unit": "cell-updates/s", "cores": r["threads"], "kind": "port",
                "sample": r["sample"]}
    import numpy as np
    from oracle import ns

    n = n_full
    while n > 64 and (n ** 3) > 128 ** 3:
        n //= 2
    u = ns.randomfield(n, 1.0, kpeak, 0)
    lst = [ns.Les(c=c, kind=k) for c, k in les if n // c >= 4]
    t0 = time.perf_counter()
    steps = 0
    while True:
        u, _, _ = ns.dnsaid_rk4(u, visc, 1.0, 0.3, 1, lst)
        steps += 1
        if time.perf_counter() - t0 > budget_s * 0.5 or steps >= 3:
            break
    el = time.perf_counter() - t0
    return {"value": n ** 3 * steps / el, "unit": "cell-updates/s", "cores": 1, "kind": "port",
            "sample": f"NumPy oracle, {steps} RK4 step(s) of a {n}^3 DNS with LES ratios "
                      f"{[c for c, _ in les]} (same physics, grid reduced to bound CPU time), single thread"}


SERVE_SIZES = (64, 96, 128, 192, 256)
SERVE_VISC = (1 / 1000, 1 / 2000, 1 / 4000)


def forms_errors(n, les, kpeak, visc, nsteps, stream):
    """Precision comparison of the 512^3 config: the FP32 form against the FP64
    plain path from the same initial field with the same fixed time step,
    after `nsteps` RK4 steps: relative L2 of the velocity, of the exact closure
    of each LES grid (stage 1 of the last step) and of the energy spectrum."""
    import numpy as np

    from exactclosure_gb300 import navierstokes as NS

    ca = NS.Case(n, 1.0, visc, 0.3, precision=0, les=les, stream=stream.cuda_stream)
    ca.init_random(kpeak, 1.0, seed=0)
    u0 = ca.velocity()
    ca.step(1)
    dt = ca.time()[1]
    ca.set_velocity(u0)
    cb = NS.Case(n, 1.0, visc, 0.3, precision=1, les=les, stream=stream.cuda_stream)
    cb.set_velocity(u0)
    ca.step(nsteps, dt=dt)
    cb.step(nsteps, dt=dt)
    ca.sync()
    cb.sync()

    def rel(a, b):
        return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))

    out = {"steps": nsteps, "dt": dt,
           "velocity": rel(cb.velocity(), ca.velocity()),
           "closure": {f"{n // c}^3 {k}": rel(cb.les(i, "closure"), ca.les(i, "closure"))
                       for i, (c, k) in enumerate(les)},
           "spectrum": rel(cb.spectrum(), ca.spectrum()),
           "exact_les_vs_filtered_dns_f32": {f"{n // c}^3 {k}": cb.errors(i)[0] for i, (c, k) in enumerate(les)},
           "note": "FP32 form vs FP64 plain path, same initial field and fixed dt; relative L2"}
    ca.close()
    cb.close()
    return out


def c1_section(nsteps=100, cpu=True):
    """The plain-method configuration: DNS 128^3 FP64, nu = 1/2000, seeded
    peak spectrum k0 = 4 with unit energy, RK4 at CFL 0.3 for 100 steps with
    the exact closure every stage for a 32^3 volume-average LES (ratio 4).
    All 100 steps are timed with CUDA events on the case's stream (inputs fit
    in L2 at this size: 50 MB per vector field)."""
    import torch

    from exactclosure_gb300 import navierstokes as NS

    n, les = 128, [(4, "volume")]
    stream = torch.cuda.Stream()
    cs = NS.Case(n, 1.0, 1 / 2000, 0.3, precision=0, les=les, stream=stream.cuda_stream)
    cs.init_random(4.0, 1.0, seed=0)
    cs.step(3)  # warm-up: graph capture
    cs.sync()
    cs.init_random(4.0, 1.0, seed=0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    cs.step(nsteps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    cs.sync()
    e_exact, e_nomo = cs.errors(0)
    out = {"metric": "cell-updates/s", "value": n ** 3 * nsteps / (ms / 1e3), "unit": "cell-updates/s",
           "dtype": "f64", "steps": nsteps, "ms_per_step": ms / nsteps, "t_end": cs.time()[0],
           "config": {"workload": "DNS 128^3 FP64 RK4 CFL 0.3, nu 1/2000, k0 4, exact closure every stage for "
                                  "LES 32^3 volume ratio 4", "timing": "CUDA events around all steps",
                      "l2": "fields fit in L2 at this size"},
           "les_errors_vs_filtered_dns": {"exact": e_exact, "nomodel": e_nomo}}
    cs.close()
    if cpu:
        try:
            from oracle import cpu_ref

            r = cpu_ref.time_stages(n, les, 4.0, 1 / 2000, budget_s=6.0, max_stages=40)
            out["cpu_baseline"] = {"value": r["cell_updates_per_s"], "unit": "cell-updates/s", "cores": r["threads"],
                                   "kind": "port", "sample": r["sample"]}
        except Exception as ex:
            out["cpu_baseline"] = {"value": None, "sample": f"failed: {ex}"}
    return out


def rhs_section(args, launches=4):
    """The RHS sweep alone on the workload's seeded field (no stepping):
    `launches` launches timed with CUDA events; a small command for profiling
    one launch of the sweep at full size."""
    import torch

    from exactclosure_gb300 import navierstokes as NS
    from exactclosure_gb300._lib import call
    import ctypes as C

    prec = 0 if args.precision == "f64" else 1
    n = args.n
    dtype = torch.float64 if prec == 0 else torch.float32
    stream = torch.cuda.Stream()
    cs = NS.Case(n, 1.0, args.visc, 0.3, precision=prec, stream=stream.cuda_stream)
    cs.init_random(args.kpeak, 1.0, seed=0)
    cs.sync()
    du = torch.empty((3, n, n, n), dtype=dtype, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(launches):
        call("exc_tensordivergence", prec, n, 1.0, args.visc, C.c_void_p(cs.device_ptr()), C.c_void_p(du.data_ptr()),
             0, C.c_void_p(stream.cuda_stream))
    e1.record(stream)
    torch.cuda.synchronize()
    cs.close()
    return {"n": n, "precision": args.precision, "launches": launches, "ms_per_launch": e0.elapsed_time(e1) / launches}


def large_and_learned_sections(n=1024, nsteps=300, every=10, do_large=True, do_learned=True, train_steps=300,
                               les_steps=200, peaks_json=None):
    """The large DNS-aided LES and the learned closure trained on its data.

    Large: DNS at 1024^3 in FP32 (FP64 spectral divide), nu = 1/8000, k0 = 8,
    exact closure at every RK4 stage for 64^3 and 128^3 LES grids with both
    the volume and the face filter; (filtered velocity, exact closure) pairs
    of the 64^3 volume LES written every `every` steps (raw binary + JSON
    header).  A bounded sample of the 500-step run: `nsteps` steps.

    Learned: 3 BF16 conv layers 3->32->32->3, 3^3 periodic, GELU, FP32
    accumulation, Adam lr 1e-3, batch 8 snapshots of 64^3 x 3, trained on the
    pairs the large run wrote (read back from its files): the first 80% of
    the run for training, the last 20% held out (a later part of the run).
    Then the net drives a 64^3 LES in lockstep with the same DNS from its
    filtered state for `les_steps` steps (a sample of the 2000 steps), with
    the no-model fallback armed; errors against the filtered DNS beside the
    no-model and exact-closure LES."""
    import tempfile

    import numpy as np
    import torch

    from exactclosure_gb300 import learned as LN
    from exactclosure_gb300 import navierstokes as NS
    from exactclosure_gb300 import snapshots

    les = [(n // 64, "volume"), (n // 128, "volume"), (n // 64, "face"), (n // 128, "face")]
    stream = torch.cuda.Stream()
    cs = NS.Case(n, 1.0, 1 / 8000, 0.3, precision=1, les=les, stream=stream.cuda_stream)
    cs.init_random(8.0, 1.0, seed=0)
    cs.step(1)
    cs.sync()
    large = learned = None
    nsnap = max(1, nsteps // every)
    with tempfile.TemporaryDirectory() as td:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hp = snapshots.write_pairs(cs, 0, td, nsnap=nsnap, every=every, stem="large")
        cs.sync()
        el = time.perf_counter() - t0
        nbytes = sum(f.stat().st_size for f in Path(td).iterdir())
        nfiles = len(list(Path(td).glob("large_*.bin")))
        if do_learned:
            U_np, M_np, header = snapshots.read_pairs(hp)
    steps = nsnap * every
    if do_large:
        errs = {f"{n // c}^3 {k}": cs.errors(i)[0] for i, (c, k) in enumerate(les)}
        large = {"metric": "cell-updates/s", "value": n ** 3 * steps / el, "unit": "cell-updates/s", "dtype": "f32",
                 "steps": steps, "seconds": el,
                 "config": {"workload": f"DNS {n}^3 FP32 (FP64 spectral divide), nu 1/8000, k0 8, exact closure every "
                                        f"RK4 stage for LES 64^3 and 128^3 x volume/face, pairs every {every} steps",
                            "sample": f"{steps} of the 500 steps"},
                 "snapshots": {"files": nfiles, "bytes": nbytes, "header": Path(hp).name},
                 "exact_closure_error_vs_filtered_dns": errs,
                 "timing": "wall clock around the stepping and the snapshot writes (host copies included)"}
    if do_learned:
        S = U_np.shape[0]
        ntr = max(1, int(round(0.8 * S)))
        U = torch.tensor(U_np, dtype=torch.float32, device="cuda")
        M = torch.tensor(M_np, dtype=torch.float32, device="cuda")
        del U_np, M_np
        net = LN.Net(seed=1)
        LN.train(net, U[:ntr], M[:ntr], steps=3)  # warm-up (also fixes the scales)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        losses = LN.train(net, U[:ntr], M[:ntr], steps=train_steps, batch=8, lr=1e-3)
        torch.cuda.synchronize()
        tel = time.perf_counter() - t0
        m = n // les[0][0]
        flop_fwd = 2 * 27 * (3 * 32 + 32 * 32 + 32 * 3) * m ** 3  # per sample, useful channels
        flops = 3 * flop_fwd * 8 * train_steps  # forward + input and weight gradients
        pred = torch.empty_like(U[ntr:])
        net.forward(U[ntr:].contiguous(), pred)
        torch.cuda.synchronize()
        e_closure = float((pred - M[ntr:]).double().norm() / M[ntr:].double().norm())
        pred_tr = torch.empty_like(U[:ntr])
        net.forward(U[:ntr].contiguous(), pred_tr)
        torch.cuda.synchronize()
        e_closure_train = float((pred_tr - M[:ntr]).double().norm() / M[:ntr].double().norm())
        del pred, pred_tr
        # a posteriori: the learned LES in lockstep with the DNS, fallback armed
        cs.reset_les()
        cs.attach_net(0, net)
        e0 = 0.5 * float(U[-1].double().pow(2).sum()) / m ** 3
        cs.set_fallback(0, 0.0, 4.0 * e0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cs.step(les_steps)
        cs.sync()
        les_el = time.perf_counter() - t0
        achieved = flops / tel / 1e12
        peak = (peaks_json or {}).get("bf16_tflops")
        times = header["times_after_step"]
        learned = {
            "metric": "training samples/s", "value": 8 * train_steps / tel, "unit": "samples/s",
            "dtype": "bf16 (fp32 accumulate)",
            "config": {"workload": f"conv 3->32->32->3 on {m}^3 x 3, batch 8, Adam lr 1e-3, {train_steps} steps; "
                                   f"trained on the {n}^3 run's pairs (files), {ntr} of {S} snapshots "
                                   f"(t <= {times[ntr - 1]:.4f}), held out the last {S - ntr} (t >= {times[ntr]:.4f})"
                       if S > ntr else f"{S} snapshots"},
            "tensor": {"achieved_tflops": achieved, "peak_tflops": peak, "frac": (achieved / peak) if peak else None,
                       "note": "useful-channel flops (3->32->32->3) of forward + both gradients; BF16 on tcgen05 "
                               "(32-channel-input convolutions, tensor-memory accumulators) and mma.sync (the rest)"},
            "loss_first_last": [losses[0], losses[-1]],
            "closure_error_vs_exact": {"held_out_later_snapshots": e_closure, "training_snapshots": e_closure_train,
                                       "no_model": 1.0},
            "les_in_lockstep": {"steps": les_steps, "sample": f"{les_steps} of the 2000 steps", "seconds": les_el,
                                "error_vs_filtered_dns": {"learned": cs.les_error(0, "learned"),
                                                          "nomodel": cs.les_error(0, "nomodel"),
                                                          "exact": cs.les_error(0, "exact")},
                                "fallback_band": [0.0, 4.0 * e0], "fallback_engaged": cs.fallback_engaged(0)}}
        net.close()
        del U, M
    cs.close()
    torch.cuda.empty_cache()
    return large, learned


def burgers_section(nsample=1000, grids=(300, 900, 2700), cpu=True, tstop=0.1):
    """The reference's Burgers DNS-aided LES setup (src/Burgers.jl:235-265):
    nh = 13500, 1000 samples, nu = 5e-4, k0 = 10, E = 2, Gaussian LES filter
    Delta = 2H, t = 0.1 with CFL 0.3, forward Euler, four LES per grid.  One
    kernel launch advances every sample to t = 0.1 (about 1470 steps each)."""
    import torch

    from exactclosure_gb300 import burgers as GB

    L, nh, visc = 2 * math.pi, 13500, 5e-4
    b = GB.Batch(GB.Grid(L, nh), nsample, visc)
    b.randomfield(10, 2.0, 1)
    runs = {}
    total_units, total_s = 0.0, 0.0
    for nH in grids:
        b.restart()
        b.les_setup(GB.Grid(L, nH), 2.0, "gaussian")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.advance(tstop, 0.3)
        el = time.perf_counter() - t0
        _, steps = b.time()
        units = float(steps.sum()) * nh
        total_units += units
        total_s += el
        err = b.errors()
        runs[str(nH)] = {"seconds": el, "cell_updates_per_s": units / el, "sample_steps": int(steps.sum()),
                         "errors_vs_filtered_dns": {k: err[k] for k in ("nomodel", "class_m", "class_p", "swapfil")}}
    b.close()
    out = {"metric": "cell-updates/s", "value": total_units / total_s, "unit": "cell-updates/s", "dtype": "f64",
           "config": {"workload": f"1-D Burgers dns_aided_les, nh {nh}, {nsample} samples, LES grids "
                                  f"{list(grids)}, Gaussian Delta = 2H, t = 0.1, CFL 0.3",
                      "timing": "wall clock around each advance call (one launch runs every sample to t = 0.1)"},
           "per_grid": runs}
    if cpu:
        try:
            from oracle import build_cpu, burgers as OB, cpu_ref

            build_cpu.build()
            cores = os.cpu_count() or 1
            ns = 2 * cores
            u0 = OB.randomfields(ns, nh, L, 10, 2.0, 1)
            _, les, dbl = OB.kernels(nh, grids[0], L, 2.0, "gaussian")
            t0 = time.perf_counter()
            _, _, _, steps = cpu_ref.burgers_dnsaid(u0, grids[0], visc, L, les[1], dbl[1], 0.1, 0.3)
            el = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": float(steps.sum()) * nh / el, "unit": "cell-updates/s", "cores": cores,
                                   "kind": "port", "sample": f"{ns} samples of nh {nh} to t = 0.1 with LES grid "
                                                             f"{grids[0]} (C/OpenMP restatement, {el:.1f} s)"}
        except Exception as ex:  # the baseline is reported, never required
            out["cpu_baseline"] = {"value": None, "sample": f"failed: {ex}"}
    return out


def serve_requests(nreq=96, rate=20.0, seed=0, nsteps=200):
    """The serving stream: seeded Poisson arrivals (mean `rate` per second),
    grid sizes uniform over SERVE_SIZES, viscosities uniform over SERVE_VISC."""
    import numpy as np

    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, nreq))
    n = rng.choice(SERVE_SIZES, nreq)
    v = rng.choice(SERVE_VISC, nreq)
    return [dict(t=float(t[i]), n=int(n[i]), visc=float(v[i]), seed=1000 + i, nsteps=nsteps) for i in range(nreq)]


def _latency_summary(res, nreq):
    import numpy as np

    lat = np.array([r["t_finish"] - r["t_submit"] for r in res])
    t_first = min(r["t_submit"] for r in res)
    t_last = max(r["t_finish"] for r in res)
    cells = sum(r["n"] ** 3 * r["nsteps"] for r in res)
    return {"value": cells / (t_last - t_first), "unit": "cell-updates/s", "solves": len(res),
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "makespan_s": t_last - t_first}


def serve_stream(precision=1, nreq=96, rate=20.0, nsteps=200, max_active_per_size=0):
    """Replay the stream in real time through the serving form; returns
    aggregate cell-updates/s and solve-latency percentiles (latency = finish
    on the GPU clock minus arrival)."""
    from exactclosure_gb300 import serving

    reqs = serve_requests(nreq, rate, nsteps=nsteps)
    sv = serving.Server(precision=precision, mem_fraction=0.6, max_active_per_size=max_active_per_size)
    # warm the per-size batches (allocation, autotuning, graph capture) untimed
    for n in SERVE_SIZES:
        sv.submit(n, 1 / 1000, 1, seed=1)
    sv.drain()
    sv.poll()
    ids = {}
    done = {}
    i = 0
    t0 = time.perf_counter()
    while len(done) < nreq:
        now = time.perf_counter() - t0
        while i < nreq and reqs[i]["t"] <= now:
            q = reqs[i]
            rid = sv.submit(q["n"], q["visc"], q["nsteps"], seed=q["seed"], kpeak=4.0)
            ids[rid] = i
            i += 1
        active, queued = sv.tick()
        for r in sv.poll():
            if r["id"] in ids:
                done[r["id"]] = r
        if active == 0 and queued == 0 and i < nreq:
            time.sleep(max(0.0, min(0.01, reqs[i]["t"] - (time.perf_counter() - t0))))
    st = sv.stats()
    sv.close()
    out = _latency_summary(list(done.values()), nreq)
    out.update({"ticks": st["ticks"], "chunks": st["chunks"],
                "admission": f"at most {max_active_per_size} active solves per grid size" if max_active_per_size
                else "every request admitted as memory and slots allow",
                "dtype": "f32 (FP64 spectral divide and diagnostics)" if precision == 1 else "f64",
                "stream": f"{nreq} solves, Poisson arrivals {rate}/s (seed 0), n in {list(SERVE_SIZES)}, "
                          f"visc in {{1/1000, 1/2000, 1/4000}}, {nsteps} RK4 steps each"})
    return out


def plain_fp64_stream(nreq=96, rate=20.0, nsteps=200):
    """The same stream through the plain FP64 path: one solve at a time
    through the case API (no batching, no overlap), in arrival order, each
    started when it has arrived and the previous solve has finished (seeded
    initial field on the GPU, 200 RK4 steps, device synchronised).  Cases are
    created and their step graphs captured per (size, viscosity) before the
    stream starts.  Latency = finish minus arrival."""
    import torch

    from exactclosure_gb300 import navierstokes as NS

    reqs = serve_requests(nreq, rate, nsteps=nsteps)
    stream = torch.cuda.Stream()
    cases = {}
    for q in reqs:
        key = (q["n"], q["visc"])
        if key not in cases:
            cs = NS.Case(q["n"], 1.0, q["visc"], 0.3, precision=0, stream=stream.cuda_stream)
            cs.init_random(4.0, 1.0, 1)
            cs.step(1)
            cs.sync()
            cases[key] = cs
    res = []
    t0 = time.perf_counter()
    for q in reqs:
        now = time.perf_counter() - t0
        if now < q["t"]:
            time.sleep(q["t"] - now)
        cs = cases[(q["n"], q["visc"])]
        cs.init_random(4.0, 1.0, q["seed"])
        cs.step(q["nsteps"])
        cs.sync()
        res.append({"t_submit": q["t"], "t_finish": time.perf_counter() - t0, "n": q["n"], "nsteps": q["nsteps"]})
    for cs in cases.values():
        cs.close()
    torch.cuda.empty_cache()
    out = _latency_summary(res, nreq)
    out.update({"dtype": "f64", "path": "case API (exc_case_*), one solve at a time in arrival order",
                "stream": f"{nreq} solves, Poisson arrivals {rate}/s (seed 0), n in {list(SERVE_SIZES)}, "
                          f"visc in {{1/1000, 1/2000, 1/4000}}, {nsteps} RK4 steps each"})
    return out


def workload_config(args, world=1):
    """The workload's `config` object, identical on both arms."""
    les = les_list(args.les)
    n = args.n
    return {"workload": f"DNS {n}^3 RK4 (4 FFT projections/step) + exact closure at every stage "
                        f"for LES {', '.join(f'{n // c}^3 {k} ratio {c}' for c, k in les)}",
            "n": n, "visc": args.visc, "kpeak": args.kpeak, "cfl": 0.3, "les": args.les,
            "l2": "inputs larger than L2 (each field >= 0.5 GB)",
            "parallelism": f"replicas x{world}"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    les = les_list(args.les)
    from oracle import cpu_ref

    if cpu_ref.available():
        # one "step" of the reference arm = one RK4 stage of the full workload
        # (a quarter of an RK4 step) on all host threads
        cs = cpu_ref.timing_case(args.n, les, args.visc, args.kpeak)
        for s in range(args.warmup):
            cs.stage(1 + s % 3)
        t0 = time.perf_counter()
        for s in range(args.steps):
            cs.stage(1 + s % 3)
        el = time.perf_counter() - t0
        cs.close()
        v = args.n ** 3 * (args.steps / 4.0) / el
        info = {"cores": cpu_ref.lib().cref_threads(), "kind": "port",
                "sample": f"C/OpenMP restatement of the path, {args.steps} RK4 stages of the {args.n}^3 DNS with "
                          f"LES {args.les} (one stage per step), all host threads"}
    else:
        vals = []
        for i in range(args.warmup + args.steps):
            r = cpu_sample(args.n, les, args.kpeak, args.visc, budget_s=8.0)
            if i >= args.warmup:
                vals.append(r["value"])
            info = r
        v = sum(vals) / len(vals)
    line = {
        "impl": "reference", "metric": "cell-updates/s", "value": v, "unit": "cell-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded spectral initial condition)",
        "config": workload_config(args, int(os.environ.get("WORLD_SIZE", "1"))),
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": info["cores"], "kind": info["kind"],
                         "sample": info["sample"]},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference Julia path unavailable (no Julia on this box); timed the project's CPU restatement",
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import numpy as np
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__  # noqa: F401  (paths)
    from exactclosure_gb300 import _lib, replicas  # noqa: F401
    from exactclosure_gb300 import navierstokes as NS

    if args.only:
        pk = measured_peaks()
        fn = {"burgers": lambda: burgers_section(args.burgers_samples, cpu=not args.no_cpu, tstop=args.burgers_tstop),
              "large": lambda: large_and_learned_sections(nsteps=args.large_steps, do_learned=False)[0],
              "learned": lambda: large_and_learned_sections(nsteps=args.large_steps, do_large=False,
                                                            train_steps=args.learned_steps,
                                                            les_steps=args.learned_les_steps, peaks_json=pk)[1],
              "c1": lambda: c1_section(cpu=not args.no_cpu),
              "rhs": lambda: rhs_section(args)}[args.only]
        print(json.dumps({args.only: fn()}))
        return
    if args.serve_only:
        served = serve_stream(precision=1, nsteps=args.serve_steps)
        served["bounded_admission"] = serve_stream(precision=1, nsteps=args.serve_steps, max_active_per_size=2)
        if not args.no_fp64_stream:
            plain = plain_fp64_stream(nsteps=args.serve_steps)
            served["plain_fp64_same_stream"] = plain
            served["served_over_plain_fp64"] = served["value"] / plain["value"]
            served["p99_plain_over_served"] = plain["p99_latency_s"] / served["p99_latency_s"]
        print(json.dumps({"serving": served}))
        return
    prec = 0 if args.precision == "f64" else 1
    les = les_list(args.les)
    n = args.n
    N = n ** 3
    stream = torch.cuda.Stream()
    cs = NS.Case(n, 1.0, args.visc, 0.3, precision=prec, les=les, stream=stream.cuda_stream)
    cs.init_random(args.kpeak, 1.0, seed=rank)
    cs.step(args.warmup)
    cs.sync()
    launches = cs.launches_per_step()

    def barrier():
        if world > 1:
            dist.barrier()

    # ---- device-resident timed region ----
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        cs.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = e0.elapsed_time(e1)
    cs.sync()
    ms_max = replicas.slowest(ms, device="cuda")
    value = replicas.job_rate(N * args.steps, ms_max / 1000.0, world)

    # ---- end to end through the public API with host buffers ----
    e2e = None
    if not args.no_e2e:
        u_host = torch.empty((3, n, n, n), dtype=torch.float64, pin_memory=True)
        u_np = u_host.numpy()
        u_np[...] = cs.velocity()
        out_host = torch.empty((3, n, n, n), dtype=torch.float64, pin_memory=True).numpy()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cs.set_velocity(u_np)  # h2d of the initial state (pinned)
        metric_bytes = 0
        for _ in range(args.steps):
            cs.step(1)
            tcur, dtcur = cs.time()  # d2h of the step's clock and dt (host loop of dnsaid_project)
            metric_bytes += 16
        cs.get_velocity_into(out_host)  # d2h of the final state
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        barrier()
        el = replicas.slowest(el, device="cuda")
        state_bytes = 3 * N * 8
        e2e = {"value": replicas.job_rate(N * args.steps, el, world), "unit": "cell-updates/s",
               "h2d_bytes_per_step": state_bytes / args.steps,
               "d2h_bytes_per_step": (state_bytes + metric_bytes) / args.steps,
               "note": "initial state uploaded and final state downloaded (pinned host buffers) inside the "
                       "timed region, amortised per step; each step reads back t and dt like the reference's "
                       "host loop"}

    # ---- roofline of the dominant kernel, timed live ----
    roof = None
    if rank == 0:
        roof = roofline(cs, NS, n, prec, args, stream)

    # ---- the other precision on the same workload, and the serving stream ----
    forms = None
    serving_line = None
    if rank == 0 and world == 1:
        cs.close()
        torch.cuda.empty_cache()
        if not args.no_forms:
            other = 1 - prec
            c2 = NS.Case(n, 1.0, args.visc, 0.3, precision=other, les=les, stream=stream.cuda_stream)
            c2.init_random(args.kpeak, 1.0, seed=rank)
            c2.step(max(1, args.warmup))
            c2.sync()
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            f0.record(stream)
            c2.step(args.steps)
            f1.record(stream)
            torch.cuda.synchronize()
            fms = f0.elapsed_time(f1)
            c2.sync()
            forms = {("f32" if other == 1 else "f64"): {
                "value": N * args.steps / (fms / 1e3), "unit": "cell-updates/s", "ms_per_step": fms / args.steps,
                "note": "same workload; f32 = stencil/filter/RK in FP32 with FP64 spectral divide and diagnostics"}}
            c2.close()
            torch.cuda.empty_cache()
            if args.forms_steps > 0:
                try:
                    forms["f32_vs_f64_error"] = forms_errors(n, les, args.kpeak, args.visc, args.forms_steps, stream)
                except Exception as ex:
                    forms["f32_vs_f64_error"] = {"error": str(ex)}
                torch.cuda.empty_cache()
        if not args.no_serve:
            try:
                served = serve_stream(precision=1)
                served["bounded_admission"] = serve_stream(precision=1, max_active_per_size=2)
                plain = plain_fp64_stream()
                served["plain_fp64_same_stream"] = plain
                served["served_over_plain_fp64"] = served["value"] / plain["value"]
                served["p99_plain_over_served"] = plain["p99_latency_s"] / served["p99_latency_s"]
                serving_line = served
            except Exception as ex:
                serving_line = {"error": str(ex)}

    large = learned = c1 = None
    if rank == 0 and world == 1 and not args.no_c1:
        try:
            c1 = c1_section(cpu=not args.no_cpu)
        except Exception as ex:
            c1 = {"error": str(ex)}
    if rank == 0 and world == 1 and not (args.no_large and args.no_learned):
        try:
            large, learned = large_and_learned_sections(nsteps=args.large_steps, do_large=not args.no_large,
                                                        do_learned=not args.no_learned,
                                                        train_steps=args.learned_steps,
                                                        les_steps=args.learned_les_steps,
                                                        peaks_json=measured_peaks())
        except Exception as ex:
            large = learned = {"error": str(ex)}
    burgers = None
    if rank == 0 and world == 1 and not args.no_burgers:
        try:
            burgers = burgers_section(cpu=not args.no_cpu)
        except Exception as ex:
            burgers = {"error": str(ex)}

    # ---- CPU baseline ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu = cpu_sample(n, les, args.kpeak, args.visc)
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "cell-updates/s", "cores": 0, "kind": "port", "sample": f"failed: {ex}"}

    if rank == 0:
        line = {
            "metric": "cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
            "data": "synthetic (seeded spectral initial condition, E(k) ~ k^4 exp(-2(k/k0)^2), unit energy)",
            "config": workload_config(args, world),
            "gpu_launches": launches * args.steps,
            "clocks": clk.summary(),
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "forms": forms,
            "c1": c1,
            "serving": serving_line,
            "burgers": burgers,
            "large": large,
            "learned": learned,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


# Algorithmic FP64 operations per cell of one RHS sweep (stresstensor +
# tensordivergence, src/N.jl:94-160), an FMA counted as two: each of the
# three off-diagonal stresses 1/4 (u_i + u_i')(u_j + u_j') - (nu/h)(du_i + du_j)
# takes 9 (two sums, the product, three differences and sums, a multiply and
# an FMA), each diagonal stress 6; the divergence of each of the three
# components takes three differences, two sums and the 1/h scaling (6).
RHS_FLOPS_PER_CELL = 3 * 9 + 3 * 6 + 3 * 6


def dgemm_peak(reps=5, size=8192):
    """The FP64 ceiling of this GPU, measured: cuBLAS DGEMM size^3, best of
    `reps` launches (CUDA events), with the SM clock sampled meanwhile."""
    import torch

    a = torch.randn(size, size, dtype=torch.float64, device="cuda")
    b = torch.randn(size, size, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = None
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(reps):
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record()
            torch.matmul(a, b)
            f1.record()
            torch.cuda.synchronize()
            t = f0.elapsed_time(f1) / 1e3
            best = t if best is None else min(best, t)
    del a, b
    torch.cuda.empty_cache()
    return 2 * size ** 3 / best / 1e12, clk.summary(), f"cuBLAS DGEMM {size}^3, best of {reps} (CUDA events), this run"


def roofline(cs, NS, n, prec, args, stream):
    """The dominant kernel of the step, the RHS sweep (stresstensor +
    tensordivergence), timed alone with CUDA events on its own stream, on the
    case's device velocity.  In FP64 it is bound by the FP64 pipe: achieved
    = algorithmic FP64 operations per launch / launch time, against the DGEMM
    rate measured in the same run; its HBM figures sit beside.  In FP32 it
    is bound by HBM: achieved = algorithmic bytes / launch time."""
    import torch

    hbm, src = peaks()
    w = 8 if prec == 0 else 4
    dtype = torch.float64 if prec == 0 else torch.float32
    ptr = cs.device_ptr()
    N = n ** 3
    du = torch.empty((3, n, n, n), dtype=dtype, device="cuda")
    import ctypes as C
    from exactclosure_gb300._lib import call

    def launch():
        call("exc_tensordivergence", prec, n, 1.0, args.visc, C.c_void_p(ptr), C.c_void_p(du.data_ptr()), 0,
             C.c_void_p(stream.cuda_stream))

    for _ in range(3):
        launch()
    reps = 10
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        launch()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    del du
    alg_bytes = 6 * N * w  # read u (3 words), write du (3 words) per cell
    gbs = alg_bytes / (ms / 1e3) / 1e9
    flops = RHS_FLOPS_PER_CELL * N
    traffic = None
    tp = ROOT / "profiles" / "rhs_traffic.json"
    if tp.exists():
        d = json.loads(tp.read_text())
        key = f"{'f64' if prec == 0 else 'f32'}_{n}"
        if key in d:
            traffic = d[key]
    hbm_part = {"achieved": gbs, "peak": hbm, "peak_source": src, "unit": "GB/s", "frac": gbs / hbm,
                "algorithmic_bytes_per_launch": alg_bytes}
    common = {"kernel": "rhs_kernel (stress + divergence sweep)", "ms_per_launch": ms, "traffic": traffic,
              "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum of one launch at this size (ncu), "
                              "bytes per launch"}
    if prec == 0:
        dgemm, dclk, dsrc = dgemm_peak()
        ach = flops / (ms / 1e3) / 1e12
        return {**common, "bound": "fp64", "achieved": ach, "peak": dgemm, "peak_source": dsrc,
                "peak_clocks": dclk, "unit": "TFLOP/s", "frac": ach / dgemm,
                "algorithmic_flops_per_launch": flops, "flops_per_cell": RHS_FLOPS_PER_CELL,
                "hbm": hbm_part}
    return {**common, "bound": "hbm", **hbm_part,
            "fp32": {"achieved_tflops": flops / (ms / 1e3) / 1e12, "flops_per_cell": RHS_FLOPS_PER_CELL}}


if __name__ == "__main__":
    main()

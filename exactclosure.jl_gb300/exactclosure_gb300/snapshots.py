"""Snapshot pairs (filtered DNS velocity, exact closure) every k steps of a
DNS-aided run, written as raw little-endian binary with a JSON header.

The reference stores its fields with JLD2 (``dns_aid.jl:87-103``,
``warmup.jl:86-88``); here each snapshot is ``<stem>_<index>.bin`` holding
two float64 arrays back to back -- the filtered DNS ``ubar`` and the exact
closure ``m``, each ``3 x m^3`` words, x fastest, component slowest -- and
``<stem>.json`` describes the run and lists the files.  The pairs are taken
at stage 1 of an RK4 step, where ``m`` is the closure of that ``ubar``.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np


def write_pairs(case, les_index: int, outdir, nsnap: int, every: int, stem: str = "pairs") -> Path:
    """Step ``case`` ``nsnap * every`` times, writing one pair every ``every`` steps."""
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)
    ratio, kind = case.les_list[les_index]
    m = case.n // ratio
    files = []
    times = []
    for s in range(nsnap):
        case.step(every)
        ub = case.les(les_index, "target_last")
        mc = case.les(les_index, "closure")
        f = out / f"{stem}_{s:05d}.bin"
        with open(f, "wb") as fh:
            fh.write(np.ascontiguousarray(ub, dtype="<f8").tobytes())
            fh.write(np.ascontiguousarray(mc, dtype="<f8").tobytes())
        files.append(f.name)
        times.append(case.time()[0])
    header = {
        "format": "two little-endian float64 arrays per file: ubar then m, each [3][m][m][m], x fastest",
        "n_dns": case.n, "n_les": m, "ratio": ratio, "filter": kind, "l": case.l, "visc": case.visc,
        "every": every, "times_after_step": times, "files": files,
    }
    hp = out / f"{stem}.json"
    hp.write_text(json.dumps(header, indent=1))
    return hp


def read_pairs(header_path):
    """Load every pair listed in a header: arrays ubar, m of shape (S, 3, m, m, m)."""
    hp = Path(header_path)
    h = json.loads(hp.read_text())
    m = h["n_les"]
    cnt = 3 * m ** 3
    U, M = [], []
    for name in h["files"]:
        a = np.fromfile(hp.parent / name, dtype="<f8")
        U.append(a[:cnt].reshape(3, m, m, m))
        M.append(a[cnt:].reshape(3, m, m, m))
    return np.stack(U), np.stack(M), h

"""Autotuner of the persistent batch renderer (kz_render_batch).

Sweeps block size, resident blocks per SM (together the number of
persistent lanes: the wavefront in flight) and the lane refill period on a
sample of the jobs, keeps the fastest by CUDA-event time, and stores it in
kazen_proto_gb300/_build/autotune.json for later calls on the same machine.
"""
from __future__ import annotations

import json
import os

from . import api

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "_build", "autotune.json")

BLOCKS = (64, 128, 256)
CTAS_PER_SM = (1, 2, 4)
PERIODS = (1, 2, 4)


def tune(jobs, reps=2, save=True):
    """jobs: built batch jobs (see scenes.build_batch_scenes). Returns
    (best config dict, table of (config, ms))."""
    table = []
    for b in BLOCKS:
        for c in CTAS_PER_SM:
            for p in PERIODS:
                cfg = api.batch_config(b, c, p, use_graph=True)
                ms = min(api.render_batch(jobs, cfg)[1]["device_ms"] for _ in range(reps))
                table.append(({"block_size": b, "ctas_per_sm": c, "refill_period": p}, ms))
    best = min(table, key=lambda x: x[1])[0]
    if save:
        os.makedirs(os.path.dirname(PATH), exist_ok=True)
        with open(PATH, "w") as f:
            json.dump({"best": best, "table": [[c, ms] for c, ms in table]}, f, indent=1)
    return best, table


def load():
    """The stored best configuration, or None."""
    if not os.path.exists(PATH):
        return None
    try:
        return json.load(open(PATH))["best"]
    except Exception:
        return None


def tuned_config(use_graph=True):
    best = load() or {}
    return api.batch_config(best.get("block_size", 0), best.get("ctas_per_sm", 0), best.get("refill_period", 0),
                            use_graph)

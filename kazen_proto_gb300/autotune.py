"""Autotuner of the batch renderer (kz_render_batch).

Sweeps, on a sample of the jobs, the wavefront mode's paths in flight, block
size and refill period (iterations between generations of new paths), the
single-launch persistent mode's paths in flight and refill period, and the
megakernel mode's block size, resident blocks per SM and lane refill period;
keeps the fastest by CUDA-event time and stores it in
kazen_proto_gb300/_build/autotune.json for later calls on the same machine.
"""
from __future__ import annotations

import json
import os

from . import api

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "_build", "autotune.json")

WAVEFRONT_SIZES = (1 << 19, 1 << 20, 1 << 21, 1 << 22, 1 << 23)
WAVE_BLOCKS = (128, 256)
BLOCKS = (64, 128, 256)
CTAS_PER_SM = (1, 2, 4)
PERIODS = (1, 2, 4)


WAVE_PERIODS = (1, 2, 3)


def candidates():
    out = [{"mode": api.BATCH_WAVEFRONT, "block_size": b, "wavefront_size": w, "refill_period": p}
           for w in WAVEFRONT_SIZES for b in WAVE_BLOCKS for p in WAVE_PERIODS]
    out += [{"mode": api.BATCH_PERSISTENT, "wavefront_size": w, "refill_period": p}
            for w in WAVEFRONT_SIZES for p in WAVE_PERIODS]
    out += [{"mode": api.BATCH_MEGAKERNEL, "block_size": b, "ctas_per_sm": c, "refill_period": p}
            for b in BLOCKS for c in CTAS_PER_SM for p in PERIODS]
    return out


def config_of(c, use_graph=True):
    return api.batch_config(c.get("block_size", 0), c.get("ctas_per_sm", 0), c.get("refill_period", 0), use_graph,
                            c.get("mode", api.BATCH_WAVEFRONT), c.get("wavefront_size", 0))


def tune(jobs, reps=2, save=True):
    """jobs: built batch jobs (see scenes.build_batch_scenes). Returns
    (best config dict, table of (config, ms))."""
    table = []
    for c in candidates():
        cfg = config_of(c)
        ms = min(api.render_batch(jobs, cfg)[1]["device_ms"] for _ in range(reps))
        table.append((c, ms))
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
    return config_of(load() or {}, use_graph)

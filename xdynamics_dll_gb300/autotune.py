"""Block-shape autotuning of the mixed contact stage, with a result cache.

`tune(sim)` returns the shapes for `sim` (threads per block of the pair and
body kernels, depth of the pair kernel's candidate stage): from the cache
file when it holds an entry for the same device and workload, otherwise by
timing every candidate on the handle's own scene (xdem_sim_autotune, which
puts the state back afterwards) and recording the winner.  The workload key
is the device name, the precision, the sphere, plane and scene counts and
the grid, so a parameter sweep that keeps its shape reuses one measurement.
"""
import json
import os

from . import types as T


def _device_name():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "cuda"


def workload_key(sim):
    sc = sim.scene
    return "|".join([_device_name(), "mixed" if sim.cfg.precision == T.XDEM_MIXED else "fp64",
                     f"np={sc.np_}", f"planes={len(sc.planes)}", f"meshes={len(sc.meshes)}",
                     f"grid={'x'.join(str(g) for g in sc.grid)}", f"scenes={getattr(sim, 'nscene', 1)}"])


def tune(sim, trial_steps=10, cache=None):
    """(shapes dict, came_from_cache) for `sim`; the shapes are set on it."""
    key = workload_key(sim)
    table = {}
    if cache and os.path.exists(cache):
        with open(cache) as f:
            table = json.load(f)
    if key in table:
        t = table[key]
        sim.set_tune(**{k: t[k] for k in T.Tune.SHAPE})
        return dict(t), True
    best, cands = sim.autotune(trial_steps)
    if cache:
        table[key] = dict(best, candidates=cands)
        tmp = cache + ".tmp"
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1)
        os.replace(tmp, cache)
    return dict(best, candidates=cands), False

"""Autotuner for the launch shapes of the batched ensemble step.

Coordinate descent over the knobs of mpcd_ensemble_set_launch (event blocks per
system, run() blocks per system, colloid-finish block size, threads per colloid
of the colloid side work, resident blocks per SM of the free-flight pass): each candidate is timed over a few whole ensemble
steps (the step call synchronises, so wall time is device time plus one host
round trip), the fastest is kept, and every timing is logged.  The results do
not depend on the shapes (every sum is exact), so tuning can run on the warm-up
steps of a production run.
"""
import time

from . import ENS_AUX, ENS_EVENTS, ENS_FIN, ENS_FREE, ENS_RUN

CANDIDATES = {
    "events_blocks_per_system": (ENS_EVENTS, [(1, 32), (2, 32), (4, 32), (8, 32)]),
    "run_blocks_per_system": (ENS_RUN, [(1, 32), (2, 32), (4, 32), (8, 32)]),
    "fin_threads_per_block": (ENS_FIN, [(1, 32), (1, 64), (1, 128)]),
    "aux_threads_per_colloid": (ENS_AUX, [(1, 64), (1, 128), (1, 256)]),
    "free_blocks_per_sm": (ENS_FREE, [(2, 256), (4, 256), (8, 256)]),
}
DEFAULTS = {"events_blocks_per_system": (2, 32), "run_blocks_per_system": (4, 32), "fin_threads_per_block": (1, 128),
            "aux_threads_per_colloid": (1, 128), "free_blocks_per_sm": (4, 256)}


def _time(ens, steps):
    ens.step(1)  # captures the step graphs of the new shape (and warms them)
    t0 = time.perf_counter()
    ens.step(steps)
    return (time.perf_counter() - t0) / steps


def autotune(ens, steps=3, rounds=1):
    """Tune `ens` in place; returns {"choice": {knob: value}, "log": [...], "ms_per_step": best}."""
    choice = dict(DEFAULTS)
    log = []
    for name, (which, _) in CANDIDATES.items():
        ens.set_launch(which, *choice[name])
    best = _time(ens, steps)
    log.append({"start": dict(choice), "ms_per_step": best * 1e3})
    for _ in range(rounds):
        for name, (which, cands) in CANDIDATES.items():
            for cand in cands:
                if cand == choice[name]:
                    continue
                ens.set_launch(which, *cand)
                t = _time(ens, steps)
                log.append({"knob": name, "value": list(cand), "ms_per_step": t * 1e3})
                if t < best:
                    best, choice[name] = t, cand
            ens.set_launch(which, *choice[name])
    return {"choice": {k: list(v) for k, v in choice.items()}, "log": log, "ms_per_step": best * 1e3}

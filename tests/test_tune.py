"""The ensemble autotuner's coordinate descent on the host, against a stand-in ensemble whose
step time is a known function of the launch shapes: it keeps the fastest value of each knob,
leaves the shapes set to its choice, and logs every trial."""
import time

from brownian_gb300 import tune


class FakeEnsemble:
    # step time (s) per knob value: the fastest is (4, 32) events, (8, 32) run(), (1, 64) finish,
    # (1, 128) side work, (2, 256) free-flight blocks
    COST = {0: {(1, 32): 3, (2, 32): 2, (4, 32): 0, (8, 32): 1},
            1: {(1, 32): 2, (2, 32): 2, (4, 32): 1, (8, 32): 0},
            2: {(1, 32): 1, (1, 64): 0, (1, 128): 2},
            3: {(1, 64): 1, (1, 128): 0, (1, 256): 2},
            4: {(2, 256): 0, (4, 256): 1, (8, 256): 2}}

    def __init__(self):
        self.shape = {}
        self.calls = []

    def set_launch(self, which, per_system=1, block=32):
        self.shape[which] = (per_system, block)
        self.calls.append((which, per_system, block))

    def step(self, n=1):
        time.sleep(n * (0.002 + 0.004 * sum(self.COST[w][v] for w, v in self.shape.items())))


def test_autotune_picks_the_fastest_shapes_and_logs_them():
    ens = FakeEnsemble()
    res = tune.autotune(ens, steps=1)
    assert res["choice"] == {"events_blocks_per_system": [4, 32], "run_blocks_per_system": [8, 32],
                             "fin_threads_per_block": [1, 64], "aux_threads_per_colloid": [1, 128],
                             "free_blocks_per_sm": [2, 256]}
    assert ens.shape == {0: (4, 32), 1: (8, 32), 2: (1, 64), 3: (1, 128), 4: (2, 256)}
    # the start and every candidate that differs from the running choice when its turn comes
    # (the default is skipped unless an earlier candidate has already replaced it), each timed
    lo = 1 + sum(len(c) - 1 for _, c in tune.CANDIDATES.values())
    assert lo <= len(res["log"]) <= lo + len(tune.CANDIDATES)
    assert all("ms_per_step" in t for t in res["log"])
    assert res["ms_per_step"] == min(t["ms_per_step"] for t in res["log"])

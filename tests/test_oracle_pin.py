"""Pin the CPU oracle to the reference itself.

tests/golden/ref_traces.json holds SHA-256 hashes of every record the
reference's own cpp/ routines wrote (oracle/ref_harness.cpp, generated by
tests/golden/make_golden.py): state after each routine, the cell number of every
particle and the occupancy of every cell for each binning, the candidate lists,
the 342-cell neighbour table.  The oracle, driven by the same sequential ran()
stream, must reproduce each record bit for bit.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle.trace import replay, sha

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TRACES = json.load(open(os.path.join(GOLDEN, "ref_traces.json")))


@pytest.mark.parametrize("case", TRACES, ids=[c["name"] for c in TRACES])
def test_oracle_matches_reference_trace(oracle_lib, case):
    recs = replay(case)
    gold = case["records"]
    assert [t for t, _ in recs] == [g[0] for g in gold]
    bad = [t for (t, b), g in zip(recs, gold) if sha(b) != g[1] or len(b) != g[2]]
    assert not bad, f"{len(bad)} records differ from the reference, first: {bad[:5]}"


def test_ran_stream_matches_reference(oracle_lib):
    for s in json.load(open(os.path.join(GOLDEN, "ran_stream.json"))):
        o = O.Oracle(L=8, n_fluid=1, n_colloid=1, mass_colloid=1.0, sig_colloid=1.0, sigma=1.0, I_colloid=1.0,
                     seed=s["seed"])
        v = o.ran(s["count"])
        assert sha(v.tobytes()) == s["sha256"], s["seed"]
        assert np.array_equal(v[:8], np.array(s["first"]))


# Philox4x32-10 known-answer vectors published with the Random123 library
# (Salmon et al., SC'11): counter, key -> output.
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_oracle_philox_known_answers(oracle_lib, ctr, key, out):
    assert O.philox(ctr, key) == out


def test_golden_cases_exercise_every_routine(oracle_lib):
    """The pinned traces must cover forces, shell kicks and wall collisions."""
    import struct
    recs = dict(replay(TRACES[2]))
    assert struct.unpack("<d", recs["setup.force/potential"])[0] > 0
    recs = dict(replay(TRACES[0]))
    assert np.frombuffer(recs["s1.run/shell_count"], dtype=np.int32).min() > 0
    moved = 0
    for nn in range(1, 3):
        for l in (1, 2):
            a = np.frombuffer(recs[f"s{nn}.l{l}.pos_mpcd/pos_fl"])
            b = np.frombuffer(recs[f"s{nn}.l{l}.collision/pos_fl"])
            moved += int((a != b).reshape(-1, 3).any(1).sum())
    assert moved > 0

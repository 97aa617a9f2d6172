"""Generate the golden traces of the reference's own C++ step.

Runs oracle/_ref/ref_harness (the reference's cpp/ routines compiled where they
lie, see oracle/Makefile target `ref`) and stores, per golden case, the SHA-256 of
every record it writes (state arrays after each routine, cell numbers and
occupancy of every binning, the candidate lists, the 342-cell neighbour table),
plus the reference's ran() stream for two seeds.  Only needs the reference
sources; run it in a checkout where they exist:

    python tests/golden/make_golden.py --ref /path/to/brownian

The tests compare the oracle's own traces of the same cases against these
hashes (tests/test_oracle_pin.py).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle.trace import parse_records, sha  # noqa: E402

GOLDEN = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

# Cases: small systems the reference runs in well under a second.
#   small_active   8^3 box, density 5, two colloids of diameter 4 with self-propulsion
#   ref_geometry   10^3 box, density 10, four colloids with the reference's own
#                  geometry (sig_colloid 2.5, diameter 0.8*sig_colloid, mass 654.1)
#   wca_cluster    12^3 box, density 2, five colloids placed by hand inside each
#                  other's WCA range so the force routine does work (the box must
#                  leave room for the reference's random placement at spacing
#                  1.3*sig_colloid, which it runs first: it loops until it fits)
CASES = [
    dict(name="small_active", crafted_colloids=None,
         params=dict(L=8, N=2560, Nc=2, n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, M=167.55,
                     sig_colloid=4.0, eps=1.0, sigma=4.0, I=0.1 * 167.55 * 16.0, v0=0.02, seed=77777,
                     nsteps=30, detail=2)),
    dict(name="ref_geometry", crafted_colloids=None,
         params=dict(L=10, N=10000, Nc=4, n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, M=654.1,
                     sig_colloid=2.5, eps=1.0, sigma=2.0, I=0.1 * 654.1 * 4.0, v0=0.0, seed=12345,
                     nsteps=10, detail=1)),
    dict(name="wca_cluster",
         crafted_colloids=[[2.0, 2.0, 2.0], [6.3, 2.1, 1.9], [2.2, 6.25, 2.05], [6.2, 6.4, 6.3], [4.1, 4.0, 6.2]],
         params=dict(L=12, N=3456, Nc=5, n_sub=10, ndt=0.1, kbt=1.0, kbt1=1.0, mass_fl=1.0, M=100.0,
                     sig_colloid=4.0, eps=1.0, sigma=4.0, I=0.1 * 100.0 * 16.0, v0=0.05, seed=4242,
                     nsteps=12, detail=2)),
]


def harness_args(p):
    return [str(p[k]) for k in ["L", "N", "Nc", "n_sub", "ndt", "kbt", "kbt1", "mass_fl", "M", "sig_colloid",
                                "eps", "sigma", "I", "v0", "seed", "nsteps", "detail"]]


def run_case(case, tmp):
    p = case["params"]
    out = os.path.join(tmp, case["name"] + ".rec")
    args = [HARNESS, "trace"] + harness_args(p) + [out]
    if case["crafted_colloids"] is not None:
        # the reference's own initial state with the colloid positions replaced
        init_out = os.path.join(tmp, case["name"] + ".init.rec")
        a0 = [HARNESS, "trace"] + harness_args(dict(p, nsteps=0, detail=0)) + [init_out]
        subprocess.run(a0, check=True, timeout=120)
        rec = dict(parse_records(init_out))
        N, Nc = p["N"], p["Nc"]
        state = np.concatenate([
            np.frombuffer(rec["init/pos_fl"], dtype=np.float64),
            np.frombuffer(rec["init/vel_fl"], dtype=np.float64),
            np.array(case["crafted_colloids"], dtype=np.float64).ravel(),
            np.frombuffer(rec["init/vel_colloid"], dtype=np.float64),
            np.frombuffer(rec["init/ang_vel_colloid"], dtype=np.float64),
        ])
        assert state.size == 3 * (2 * N + 3 * Nc)
        sf = os.path.join(tmp, case["name"] + ".state")
        state.tofile(sf)
        args.append(sf)
    subprocess.run(args, check=True, timeout=600)
    return parse_records(out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="reference checkout (the directory holding cpp/)")
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={a.ref}"], check=True)
    with tempfile.TemporaryDirectory() as tmp:
        traces = []
        for case in CASES:
            recs = run_case(case, tmp)
            traces.append(dict(case, records=[[t, sha(b), len(b)] for t, b in recs]))
            print(case["name"], len(recs), "records")
        with open(os.path.join(GOLDEN, "ref_traces.json"), "w") as f:
            json.dump(traces, f, indent=1)
        streams = []
        for seed in (77777, -7):
            out = os.path.join(tmp, f"ran{seed}.rec")
            subprocess.run([HARNESS, "ran", str(seed), "1000", out], check=True, timeout=60)
            (tag, b), = parse_records(out)
            v = np.frombuffer(b, dtype=np.float64)
            streams.append(dict(seed=seed, count=1000, sha256=sha(b), first=[float(x) for x in v[:8]]))
        with open(os.path.join(GOLDEN, "ran_stream.json"), "w") as f:
            json.dump(streams, f, indent=1)


if __name__ == "__main__":
    main()

"""Fixture generator: the reference driver's 43 test problems with oracle region counts.

The reference's own end-to-end check (main.py:213-228) runs the problems
test_ids = main.py:219 of its data file POP_mpQP1.mat through its GPU path and
prints the region-count difference to ppopt.  This script reads those 43
problems from the reference checkout (scipy.io.loadmat, as main.py:214,221
does; the fields A, b, c, F, Q, CRA, CRb, Ht of main.py:72-79) and stores
them, together with the C oracle's region count of each, in
tests/golden/pop_mpqp1_43.npz:

* ``p{i}/{A,b,c,F,Q,H,CRA,CRb}``  the raw problem (H = the file's Ht);
* ``ids``                         the 43 problem numbers in main.py's order;
* ``regions_scaled``              oracle regions after the reference's scaling
                                  (MPQPProb.process_constraints(scale_method=1)
                                  without the ppopt row reduction);
* ``regions_reduced``             oracle regions after the row reduction that
                                  restates ppopt (reduce=True) and the scaling.

Every active set up to |S| = n is enumerated.  ppopt itself is not installed
here, so the reference's own region counts for these problems (ppopt's) are
not known; these counts pin the build's device path to the oracle on the
reference's real problem mix.  Run from the repository root:

    python tests/golden/make_pop_fixture.py [path/to/POP_mpQP1.mat]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

TEST_IDS = [38, 51, 80, 41, 30, 92, 88, 99, 70, 63, 66, 93, 53, 72, 68, 9, 57, 91, 49, 13, 19, 54, 45, 58, 56, 8,
            55, 84, 67, 15, 97, 71, 3, 89, 21, 47, 79, 20, 33, 34, 74, 73, 64]
OUT = os.path.join(HERE, "pop_mpqp1_43.npz")


def main(path: str) -> None:
    import scipy.io

    from mpqpcudasolver_gb300 import host
    from mpqpcudasolver_gb300 import problems as P
    from oracle import oracle as O
    from oracle import preprocess as PP

    data = scipy.io.loadmat(path)["problem"][0]
    out = {"ids": np.array(TEST_IDS, dtype=np.int64)}
    scaled, reduced = [], []
    for i in TEST_IDS:
        pr = data[i]
        arr = {k: np.asarray(pr[k], dtype=np.float64) for k in ("A", "b", "c", "F", "Q", "CRA", "CRb")}
        arr["H"] = np.asarray(pr["Ht"], dtype=np.float64)
        for k, v in arr.items():
            out[f"p{i}/{k}"] = v
        prob = P.MPQP(arr["Q"], arr["c"].ravel(), arr["H"], arr["A"], arr["b"].ravel(), arr["F"], arr["CRA"],
                      arr["CRb"].ravel())
        prog = host.MPQPProb.from_mpqp(prob)
        prog.process_constraints(scale_method=1)
        scaled.append(O.enumerate_sets(prog.to_mpqp(), k_max=prog.num_x, nthreads=8, keep_records=False).n_region)
        # the ppopt steps restated on the host (oracle/preprocess.py), then the scaling
        status = PP.reduce_rows(prob)
        from mpqpcudasolver_gb300.solver import apply_row_status
        red = apply_row_status(prob, status)
        prog = host.MPQPProb.from_mpqp(red)
        prog.process_constraints(scale_method=1)
        reduced.append(O.enumerate_sets(prog.to_mpqp(), k_max=prog.num_x, nthreads=8, keep_records=False).n_region)
        print(i, prob.n, prob.m, prob.p, "regions", scaled[-1], reduced[-1])
    out["regions_scaled"] = np.array(scaled, dtype=np.int64)
    out["regions_reduced"] = np.array(reduced, dtype=np.int64)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/POP_mpQP1.mat")

"""Regenerates the small golden fixtures of this directory.

Run in a container that has the reference checkout and pyarrow:

    python tests/golden/make_fixtures.py /path/to/reffine

* ``students.npz``: the six int64 columns of Reffine's ``students.arrow`` fixture, built from
  ``benchmark/lib/students.csv`` the way ``benchmark/lib/students.py:1-44`` builds the Arrow
  file (columns id, hours_studied, attendance, sleep_hours, previous_scores, exam_score;
  ``gender`` dropped).
* ``runend.npz``: Reffine's ``runend.arrow`` fixture (``benchmark/lib/runend.py:1-26``): a
  run-end encoded ``x`` plus flat ``y`` and ``d``, produced through
  ``pyarrow.compute.run_end_encode`` so the run ends are Arrow's own.

The known answers the tests check against these fixtures are the reference's own test
assertions (test/src/test_reduce.cpp:58,121; test/src/test_multidim.cpp:47-54).
"""
import os
import sys

import numpy as np

COLS = ["id", "hours_studied", "attendance", "sleep_hours", "previous_scores", "exam_score"]


def main(ref_root: str):
    import pyarrow as pa
    import pyarrow.compute as pc
    import pyarrow.csv as pacsv

    here = os.path.dirname(os.path.abspath(__file__))
    tbl = pacsv.read_csv(os.path.join(ref_root, "benchmark", "lib", "students.csv"))
    arrays = {c: np.asarray(tbl.column(c).to_numpy(), dtype=np.int64) for c in COLS}
    np.savez_compressed(os.path.join(here, "students.npz"), **arrays)

    x = [1, 1, 1, 2, 2, 3, 3, 3, 3, 4]
    y = [1, 3, 7, 1, 9, 2, 3, 7, 8, 3]
    d = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9]
    ree = pc.run_end_encode(pa.array(x, type=pa.int64()))
    np.savez_compressed(os.path.join(here, "runend.npz"),
                        x_values=np.asarray(ree.values.to_numpy(), dtype=np.int64),
                        x_run_ends=np.asarray(ree.run_ends.to_numpy(), dtype=np.int32),
                        y=np.asarray(y, dtype=np.int64), d=np.asarray(d, dtype=np.int64))
    print("wrote", here)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        raise SystemExit("usage: python tests/golden/make_fixtures.py REFFINE_SRC")
    main(sys.argv[1])

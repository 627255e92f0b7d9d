"""Write tests/golden/ref_<case>.npz from runs of oracle/_ref, the reference's
own program compiled from its unmodified sources (oracle/ref/Makefile), for
every case of tests/ref_cases.py.  Each fixture holds the case, the
cosmology scalars the reference computed (D+, vfac, pnorm, ...) and what the
reference handed its output plugin (tests/ref_cases.py:reduce_outputs).

Run in the build container, where the reference's sources are:
    python tests/golden/make_ref_fixtures.py [case ...]
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refrun  # noqa: E402
from tests import ref_cases as R  # noqa: E402


def make(name):
    case = R.CASES[name]
    res = refrun.run(case)
    arrays = R.reduce_outputs(case, res)
    np.savez_compressed(R.fixture_path(name), case=json.dumps(case), scalars=json.dumps(res["scalars"]), **arrays)
    size = os.path.getsize(R.fixture_path(name))
    print(f"{name}: {res['seconds']:.1f} s, {size / 1024:.0f} KiB, keys {sorted(arrays)}")


if __name__ == "__main__":
    if not refrun.build():
        sys.exit("oracle/_ref could not be built (the reference's sources are needed)")
    for name in (sys.argv[1:] or list(R.CASES)):
        make(name)

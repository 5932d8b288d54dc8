import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_case(name):
    """A golden case: (oracle.Problem, dict of the reference's outputs)."""
    import oracle as O
    z = np.load(GOLDEN / f"{name}.npz")
    P = O.Problem(int(z["nc"]), z["rowptr"], z["colidx"], z["blocks"], z["q"], z["mu"])
    return P, {k: z[k] for k in z.files}


FIXTURE_CASES = sorted(p.stem for p in GOLDEN.glob("fixture_*.npz"))
LATTICE_CASES = sorted(p.stem for p in GOLDEN.glob("lattice_*.npz"))
CONVERGING = [c for c in FIXTURE_CASES + LATTICE_CASES if int(np.load(GOLDEN / f"{c}.npz")["info"]) == 0]


@pytest.fixture(scope="session")
def built_lib():
    from siconos_gb300 import build as B
    B.build()
    import siconos_gb300.numerics as sn
    return sn.lib()


@pytest.fixture(scope="session")
def gpu(built_lib):
    """A device context; the GPU tests fail (not skip) when none is usable."""
    from siconos_gb300.device import DeviceSolver
    try:
        d = DeviceSolver(0)
    except RuntimeError as e:
        pytest.fail(f"no usable CUDA device for a -m gpu run: {e}")
    yield d
    d.close()

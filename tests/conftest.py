import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def golden_cases():
    """The real-space Hubbard sectors dumped from the reference (cereal_*
    fixtures are cache-format pins, mom_* momentum-space sectors, mfull_*
    the momentum-space model on whole bases)."""
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(f).startswith(("cereal_", "mom_", "cur_", "all_",
                                                         "mfull_")))


def momentum_full_cases():
    """The momentum-space model on whole (N_up, N_down) bases, from the reference."""
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "mfull_*.npz")))


def all_sz_cases():
    """All spin projections (with_fixed_particle_number), from the reference."""
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "all_*.npz")))


def current_cases():
    """The current operator J_d(Q) between momentum sectors, from the reference."""
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "cur_*.npz")))


def momentum_cases():
    """The momentum-space model on total-momentum sectors, from the reference."""
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "mom_*.npz")))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    n = int(d["particles"])
    d["L"] = int(np.prod(d["dims"]))
    if "spin_projection" in d:  # all_* fixtures span every spin projection
        sz = int(d["spin_projection"])
        d["n_up"] = (n + sz) // 2
        d["n_down"] = n - d["n_up"]
    return d


@pytest.fixture(scope="session")
def mb():
    import manybody_gb300
    manybody_gb300.lib()
    return manybody_gb300


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    return torch

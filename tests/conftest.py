"""Shared test setup: import paths for the package and the oracle, the
``gpu`` marker, and fixture loaders."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "deepmd-kit_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))
GOLDEN = os.path.join(HERE, "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def deeppot_sea_params():
    """The reference's se_e2_a test model (deeppot_sea.pth weights)."""
    from dpgb import params as P

    m = golden("deeppot_sea_model")
    cfg = P.SeAConfig(sel=[46, 92], rcut=6.0, rcut_smth=0.5, neuron=[3, 6, 12], axis_neuron=2,
                      type_one_side=True, fit_neuron=[10, 10, 10])
    return P.SeAParams.from_state_dict({k: m[k] for k in m.files}, cfg)


def water_params(compressed=False):
    from dpgb import params as P

    p = P.init_params(P.water_config(), seed=1)
    if compressed:
        g = golden("water192_compressed")
        p.tables = [g[f"table_{e}"] for e in range(4)]
        p.table_info = [g[f"info_{e}"] for e in range(4)]
    return p


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")

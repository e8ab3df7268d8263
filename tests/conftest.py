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


def assert_table_close(t, ref, lower, upper, stride0, stride1, tol=1e-12):
    """Tables agree as polynomials: coefficient k of a row scaled by h^k.
    The high-order coefficients are differences of node values divided by
    h^3..h^5, so one ulp in a node value moves them by ~1e-16 / h^5; their
    contribution on the interval, a_k h^k, is what must agree."""
    nrow0 = int((upper - lower) / stride0)
    h = np.where(np.arange(t.shape[0]) < nrow0, stride0, stride1)[:, None]
    scale = np.abs(ref[:, 0::6]).max()
    for k in range(6):
        d = np.abs(t[:, k::6] - ref[:, k::6]) * h ** k
        assert d.max() <= tol * scale, (k, d.max())

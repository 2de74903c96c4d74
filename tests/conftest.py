import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libbella_gb300.so")


def golden(name):
    return os.path.join(ROOT, "tests", "golden", name)


def rb_background(d):
    """Rising-bubble backgrounds exactly as the reference computed them (from the fixture).

    Recomputing them with np.exp on another platform changes the last bit,
    and dS/dy (a difference of nearly equal numbers) turns that into ~1e-11.
    """
    from oracle import cases
    grid, prm, _, _, hn, hc, sf = cases.rising_bubble()
    hn = dict(hn)
    hc = dict(hc)
    hn["S0"] = d["hydro_n_S0"].copy()
    hc["rhoY0"] = d["hydro_c_rhoY0"].copy()
    return grid, prm, hn, hc, sf

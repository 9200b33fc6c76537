import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")

EXAMPLE_SETTINGS = {
    'sPri': 0.90924, 'sAnn': 2.887e-3, 'zAnn': 4.0, 'rInner': 0.2, 'rOuter': 1.4,
    'zExp': 12.5, 'sExp': 8.289e-3, 'kExp': 0.4816, 'softRatio': 0.0025,
    'softLimit': 20, 'hornRatio': 0.0065, 'fluenceResampling': 3,
    'energy_weights': {"0.5": 0.08196, "1.0": 0.12385, "1.5": 0.10605, "2.0": 0.08307,
                       "2.5": 0.05881, "3.0": 0.03911, "3.5": 0.02131, "4.0": 0.02426,
                       "4.5": 0.0, "5.0": 0.00881, "5.5": 0.0, "6.0": 0.00498},
}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def settings():
    import copy
    return copy.deepcopy(EXAMPLE_SETTINGS)


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    oracle.lib()
    return oracle

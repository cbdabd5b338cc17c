import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent/'golden'
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')


def golden(name):
    with np.load(GOLDEN/f'{name}.npz') as data:
        return {k: data[k] for k in data.files}


STATE = ('x', 'v', 'rotation', 'normal', 'offset', 'fn', 'fs', 'mt', 'mb')


def newton_inputs(g):
    return dict(points=g['in_points'], radii=g['in_radii'], pairs=g['in_pairs'], areas=g['in_areas'],
                masses=g['in_masses'], fixed=g['in_fixed'], contacts=g['in_contacts'],
                young=float(g['in_young']), shear=float(g['in_shear']))


@pytest.fixture
def golden_loader():
    return golden

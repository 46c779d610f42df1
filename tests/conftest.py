import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: test needs a CUDA GPU (GB300) and the built extension')
    config.addinivalue_line('markers', 'unverified(order=0): GPU test written after the last GPU run of the code '
                                       'it covers; runs after all other tests, in increasing order')


def _run_order(item):
    m = item.get_closest_marker('unverified')
    return (0, 0) if m is None else (1, int(m.kwargs.get('order', 0)))


def pytest_collection_modifyitems(config, items):
    # tests that have not yet run on a GPU go last (stable sort), those exercising
    # the least new device code first, so that under -x a failure among them
    # cannot keep the verified tests from running
    items.sort(key=_run_order)


@pytest.fixture(scope='session')
def golden_dir():
    return GOLDEN

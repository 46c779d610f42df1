import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: test needs a CUDA GPU (GB300) and the built extension')
    config.addinivalue_line('markers', 'unverified: GPU test written after the last GPU run of the code it '
                                       'covers; runs after all other tests')


def pytest_collection_modifyitems(config, items):
    # tests that have not yet run on a GPU go last (stable sort), so that under -x a
    # failure among them cannot keep the verified tests from running
    items.sort(key=lambda item: item.get_closest_marker('unverified') is not None)


@pytest.fixture(scope='session')
def golden_dir():
    return GOLDEN

import os
import sys

# Host-side linear algebra in these tests runs on one thread: on some hosts the
# multi-threaded BLAS/LAPACK paths (batched LU and solves in NumPy's OpenBLAS and
# in torch's MKL) stop making progress, and the test matrices are small.  The
# variables must be set before NumPy and torch load their BLAS.
for _v in ('OMP_NUM_THREADS', 'OPENBLAS_NUM_THREADS', 'MKL_NUM_THREADS'):
    os.environ.setdefault(_v, '1')

import pytest  # noqa: E402
import torch  # noqa: E402

torch.set_num_threads(1)
try:
    from threadpoolctl import threadpool_limits
    threadpool_limits(1)
except ImportError:
    pass

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: test needs a CUDA GPU (GB300) and the built extension')


@pytest.fixture(scope='session')
def golden_dir():
    return GOLDEN

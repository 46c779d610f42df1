"""Build the in-tree CUDA library ``libslablu_gb300.so`` for sm_103a.

    python -m slablu_gb300.build [--force]

Each ``csrc/*.cu`` file is compiled to an object in ``_build/`` (in parallel),
then linked into ``slablu_gb300/libslablu_gb300.so``.  Objects are rebuilt when
their source or any header is newer.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
BUILD = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libslablu_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
         '-Xptxas', '-warn-spills']


def nvcc():
    exe = shutil.which('nvcc')
    if exe:
        return exe
    cand = '/usr/local/cuda/bin/nvcc'
    if os.path.exists(cand):
        return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build slablu_gb300')


def _headers_mtime():
    hs = glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(ROOT, 'include', '*.h'))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src, obj, extra):
    cmd = [nvcc()] + ARCH + FLAGS + extra + ['-I', os.path.join(ROOT, 'include'), '-c', src, '-o', obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}')
    return r.stderr


def build(force=False, verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    hdr = _headers_mtime()
    jobs = []
    for src in srcs:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + '.o')
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr):
            jobs.append((src, obj))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        futs = {ex.submit(_compile, s, o, list(extra)): s for s, o in jobs}
        for f in cf.as_completed(futs):
            msg = f.result()
            if verbose and msg.strip():
                print(msg)
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + '.o') for s in srcs]
    if force or jobs or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ['-shared', '-o', LIB] + objs + ['-lcudart']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f'link failed:\n{r.stdout}\n{r.stderr}')
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose='-v' in sys.argv))

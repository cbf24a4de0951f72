"""Build recipe for the in-tree CUDA library (sm_103a only).

Compiles every ``csrc/*.cu`` with nvcc for ``sm_103a`` in parallel and links
``liblentil_gb300.so`` next to this file.  Used by ``__graft_entry__.build()``
and by ``python -m lentil_gb300._build``.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'liblentil_gb300.so')
INCLUDE = os.path.join(os.path.dirname(HERE), 'include')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
         '--expt-relaxed-constexpr', '-I' + INCLUDE]


def nvcc():
    exe = shutil.which('nvcc')
    if exe:
        return exe
    cand = '/usr/local/cuda/bin/nvcc'
    if os.path.exists(cand):
        return cand
    raise RuntimeError('nvcc not found: the lentil_gb300 CUDA library cannot be built')


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(INCLUDE, '*.h'))


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link the library; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    srcs = _sources()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + '.o')
        cmd = [cc, *ARCH, *FLAGS, *extra_flags, '-c', src, '-o', obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f'nvcc failed on {os.path.basename(src)}:\n{res.stderr}')
        if verbose and res.stderr:
            sys.stderr.write(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + '.tmp'
    cmd = [cc, *ARCH, '-shared', '-o', tmp, *objs, '-lcudart_static', '-ldl', '-lrt', '-lpthread']
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f'link failed:\n{res.stderr}')
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True,
                extra_flags=['-Xptxas', '-v'] if '--ptxas-v' in sys.argv else ()))

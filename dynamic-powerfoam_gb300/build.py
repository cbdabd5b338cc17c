"""Build ``libdpf_gb300.so`` (the C-ABI CUDA library) in-tree with nvcc.

Each ``csrc/*.cu`` is compiled for sm_103a in parallel and linked into one
shared library next to this file.  Object files go to ``_build/``.
"""
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
LIBRARY = HERE/'libdpf_gb300.so'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
# host code is not contracted into FMAs: the step driver's float64 decisions
# match the same arithmetic done in Python operation for operation
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-ffp-contract=off',
         f'-I{ROOT/"include"}', f'-I{HERE/"csrc"}']


def nvcc():
    for candidate in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if candidate and Path(candidate).exists():
            return candidate
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build libdpf_gb300.so')


def sources():
    return sorted((HERE/'csrc').glob('*.cu'))


def up_to_date():
    if not LIBRARY.exists():
        return False
    stamp = LIBRARY.stat().st_mtime
    inputs = list(sources()) + list((HERE/'csrc').glob('*.cuh')) + list((ROOT/'include').glob('*.h'))
    return all(p.stat().st_mtime <= stamp for p in inputs)


def build(force=False, verbose=False):
    """Compile every CUDA source and link the library; returns its path."""
    if not force and up_to_date():
        return LIBRARY
    compiler = nvcc()
    out = HERE/'_build'
    out.mkdir(exist_ok=True)
    jobs = []
    for src in sources():
        obj = out/(src.stem + '.o')
        cmd = [compiler, *ARCH, *FLAGS, '-c', str(src), '-o', str(obj)]
        jobs.append((cmd, obj, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    objects = []
    for cmd, obj, proc in jobs:
        text = proc.communicate()[0].decode()
        if proc.returncode != 0:
            raise RuntimeError(f'nvcc failed ({" ".join(cmd)}):\n{text}')
        if verbose and text.strip():
            print(text, file=sys.stderr)
        objects.append(str(obj))
    tmp = LIBRARY.with_suffix('.so.tmp')
    cmd = [compiler, *ARCH, '-shared', '-o', str(tmp), *objects]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if proc.returncode != 0:
        raise RuntimeError(f'link failed ({" ".join(cmd)}):\n{proc.stdout.decode()}')
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True))

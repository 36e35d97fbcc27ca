"""Builds libqgate_gb300.so (the engine's C ABI) in-tree for sm_103a.

Translation units are compiled in parallel (nvcc for the kernels, the host
compiler for the C ABI layer) and linked with nvcc against the static CUDA
runtime, so the library needs no CUDA shared libraries beyond the driver.
Objects are rebuilt only when a source or header is newer.

    python -m qgate_gb300.csrc.build [--force] [--verbose]
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
OBJDIR = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libqgate_gb300.so')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
CU_SOURCES = ['gates.cu', 'reduce.cu', 'fused.cu', 'adjoint.cu', 'batch.cu', 'noalloc.cu', 'tcstage.cu']
CXX_SOURCES = ['api.cpp', 'adjoint_host.cpp', 'tcplan.cpp']


def _cuda_home():
    home = os.environ.get('CUDA_HOME') or os.environ.get('CUDA_PATH')
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which('nvcc')
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return '/usr/local/cuda'


def _headers():
    hs = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(('.h', '.cuh'))]
    hs.append(os.path.join(ROOT, 'include', 'qgate_gb300.h'))
    return hs


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _headers())


def _run(cmd, verbose):
    if verbose:
        print(' '.join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('build failed:\n%s\n%s%s' % (' '.join(cmd), r.stdout, r.stderr))
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return r


def build(force=False, verbose=False, ptxas_verbose=False):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, 'bin', 'nvcc')
    inc = ['-I' + os.path.join(cuda, 'include'), '-I' + HERE, '-I' + os.path.join(ROOT, 'include')]
    os.makedirs(OBJDIR, exist_ok=True)
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(HERE, src)
        o = os.path.join(OBJDIR, src + '.o')
        objs.append(o)
        if force or _stale(o, s):
            cmd = [nvcc] + ARCH + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
                                   '--expt-relaxed-constexpr', '-c', s, '-o', o] + inc
            if ptxas_verbose:
                cmd += ['-Xptxas', '-v']
            jobs.append(cmd)
    for src in CXX_SOURCES:
        s = os.path.join(HERE, src)
        o = os.path.join(OBJDIR, src + '.o')
        objs.append(o)
        if force or _stale(o, s):
            cxx = os.environ.get('CXX', 'g++')
            jobs.append([cxx, '-O2', '-std=c++17', '-fPIC', '-Wall', '-fopenmp', '-c', s, '-o', o] + inc)
    outputs = []
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            outputs = list(ex.map(lambda c: _run(c, verbose), jobs))
    if jobs or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ['-shared', '-cudart', 'static', '-Xcompiler', '-fopenmp', '-o', LIB] +
             objs + ['-lgomp'], verbose)
    return LIB, outputs


if __name__ == '__main__':
    args = sys.argv[1:]
    _, outs = build(force='--force' in args, verbose='--verbose' in args,
                    ptxas_verbose='--ptxas' in args)
    if '--ptxas' in args:
        for r in outs:
            sys.stdout.write(r.stderr)
    print(LIB)

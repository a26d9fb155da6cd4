"""Build the native library in-tree: sdepy_gb300/_native/libsdepy_gb300.so.

Every translation unit under csrc/ is compiled by nvcc for sm_103a only, in
parallel, then linked with the CUDA runtime.  No cmake, no torch extension
machinery: the result is a plain C-ABI shared library loaded by ctypes.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
OUT = os.path.join(HERE, '_native')
LIB = os.path.join(OUT, 'libsdepy_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
         '-Xcompiler', '-fvisibility=hidden', '--expt-relaxed-constexpr']


def nvcc():
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'),
                 '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, '*.cu')))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(CSRC, '*.h')) + \
        [os.path.join(HERE, '..', 'include', 'sdepy_gb300.h')]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False):
    """Compile and link; returns the library path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    inc = ['-I', os.path.join(HERE, '..', 'include')]
    jobs = []
    for src in _sources():
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + '.o')
        cmd = [cc] + ARCH + FLAGS + inc + ['-c', src, '-o', obj]
        jobs.append((src, obj, cmd))

    def run(job):
        src, obj, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed on {}:\n{}\n{}'.format(
                src, r.stdout, r.stderr))
        if verbose:
            print(r.stdout, r.stderr)
        return obj

    workers = max(1, min(len(jobs), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(run, jobs))
    tmp = '{}.{}.tmp'.format(LIB, os.getpid())   # renamed into place when linked
    cmd = [cc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcudart', '-ldl']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n{}\n{}'.format(r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    import sys
    print(build(force='-f' in sys.argv, verbose='-v' in sys.argv))

"""ORACLE -- test infrastructure only.  Builds the C restatement
oracle/rng_oracle.c into oracle/_build/liboracle.so (gcc, no fused
multiply-add contraction so every operation rounds as written)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_build')
LIB = os.path.join(OUT, 'liboracle.so')
SRC = os.path.join(HERE, 'rng_oracle.c')
HDR = os.path.join(HERE, '..', 'include', 'sdepy_gb300.h')
TAB = os.path.join(HERE, 'oracle_tables.h')


def build(force=False):
    if not force and os.path.exists(LIB) and \
       os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in (SRC, HDR, TAB)):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    # (a file of this process's own, renamed into place: processes that
    # build at the same time never load a partly written library)
    tmp = '{}.{}.tmp'.format(LIB, os.getpid())
    cmd = ['gcc', '-O2', '-std=c11', '-D_DEFAULT_SOURCE', '-fPIC', '-shared',
           '-ffp-contract=off', '-fno-fast-math', SRC, '-o', tmp, '-lm']
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == '__main__':
    print(build(force=True))

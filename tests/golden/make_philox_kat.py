"""Generate tests/golden/philox_kat.json: Philox-4x32-10 known answers.

The first three vectors are the published Random123 known-answer tests
(Salmon et al., SC'11); every vector's output is recomputed here with
Triton's independent tl.philox running in the Triton CPU interpreter:

    TRITON_INTERPRET=1 python tests/golden/make_philox_kat.py
"""
import json
import os

import numpy as np
import torch
import triton
import triton.language as tl

HERE = os.path.dirname(os.path.abspath(__file__))


@triton.jit
def _philox_kernel(c0, c1, c2, c3, o0, o1, o2, o3, seed_lo, seed_hi):
    i = tl.arange(0, 4)
    a = tl.load(c0 + i)
    b = tl.load(c1 + i)
    c = tl.load(c2 + i)
    d = tl.load(c3 + i)
    seed = (seed_hi.to(tl.uint64) << 32) | seed_lo.to(tl.uint64)
    r0, r1, r2, r3 = tl.philox(seed, a, b, c, d, 10)
    tl.store(o0 + i, r0)
    tl.store(o1 + i, r1)
    tl.store(o2 + i, r2)
    tl.store(o3 + i, r3)


CASES = [
    ([0, 0, 0, 0], [0, 0]),
    ([0xffffffff]*4, [0xffffffff]*2),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]),
    ([7, 123456, 99, 5], [11, 22]),
    ([1048575, 1007, (3 << 8) | 1, 42], [0xdeadbeef, 0x01234567]),
]


def main():
    out = []
    for ctr, key in CASES:
        cs = [torch.tensor([ctr[j]]*4, dtype=torch.uint32) for j in range(4)]
        os_ = [torch.zeros(4, dtype=torch.uint32) for _ in range(4)]
        _philox_kernel[(1,)](*cs, *os_, key[0], key[1])
        out.append({'ctr': ctr, 'key': key, 'out': [int(o[0]) for o in os_]})
    with open(os.path.join(HERE, 'philox_kat.json'), 'w') as f:
        json.dump(out, f, indent=1)
    print(out)


if __name__ == '__main__':
    main()

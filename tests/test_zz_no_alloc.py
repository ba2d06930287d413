"""qcdgpu_dot_noalloc: the dot product for callers that cannot allocate
device memory (a framework owns the device heap, a serving engine reserved
its budget up front, or an allocation's synchronisation is unaffordable).

It is called through the C ABI on device arrays the test already owns and
must agree with the library's regular dot product (qcdgpu_dot), within the
FP64 reduction tolerance of the BLAS tests, on two calls in a row (the
shared 32 KB partial-sum array keeps the first call's contents), give a small
call's value after a large call, and leave the library's reduction scratch
unallocated. This file
sorts last so a run that stops at the first failure has run everything
else; it also passes on its own in a fresh process.
"""
import ctypes as C
import math
import os
import subprocess
import sys

import numpy as np
import pytest

import qcd_gb300 as q

pytestmark = pytest.mark.gpu

MAX_N = 2048 * 65536


def test_dot_noalloc_matches_regular_dot_twice(gpu):
    lib = q.lib()
    L = (16, 8, 8, 8)
    a = q.Field(L).gaussian(101)
    b = q.Field(L).gaussian(202)
    res = q.Field((2, 2, 2, 2))  # its first complex word receives the result
    expected = a.dot(b)  # the regular entry point
    scale = math.sqrt(a.norm2() * b.norm2())
    n = a.nbytes // 16  # complex doubles in the field's storage (padding is zero)
    pa, pb = lib.qcdgpu_field_data(a.h), lib.qcdgpu_field_data(b.h)
    pr = lib.qcdgpu_field_data(res.h)
    got = []
    for _ in range(2):
        assert lib.qcdgpu_dot_noalloc(pa, pb, n, pr, None) == 0, lib.qcdgpu_last_error()
        q.sync()
        r = res.store()[0, 0, 0]
        got.append(complex(r[0], r[1]))
    for g in got:
        assert abs(g - expected) <= 1e-14 * scale
    assert got[0] == got[1]  # fixed summation order


def test_dot_noalloc_other_sizes_after_a_large_call(gpu, orc):
    """a small call after a large one must not see the large call's partials:
    the large call (16^4, 786,432 complex elements) fills many chunks' slots"""
    lib = q.lib()
    big_a, big_b = q.Field((16, 16, 16, 16)).gaussian(7), q.Field((16, 16, 16, 16)).gaussian(8)
    res = q.Field((2, 2, 2, 2))
    pr = lib.qcdgpu_field_data(res.h)
    assert lib.qcdgpu_dot_noalloc(lib.qcdgpu_field_data(big_a.h), lib.qcdgpu_field_data(big_b.h),
                                  big_a.nbytes // 16, pr, None) == 0
    q.sync()
    r = res.store()[0, 0, 0]
    assert abs(complex(r[0], r[1]) - big_a.dot(big_b)) <= 1e-14 * math.sqrt(big_a.norm2() * big_b.norm2())
    L = (2, 2, 2, 2)
    av, bv = orc.gaussian_spinor(L, 5), orc.gaussian_spinor(L, 6)
    a, b = q.Field(L).load(av), q.Field(L).load(bv)
    n = a.nbytes // 16
    assert lib.qcdgpu_dot_noalloc(lib.qcdgpu_field_data(a.h), lib.qcdgpu_field_data(b.h), n, pr, None) == 0
    q.sync()
    r = res.store()[0, 0, 0]
    ref = complex(np.vdot(av[..., 0] + 1j * av[..., 1], bv[..., 0] + 1j * bv[..., 1]))
    assert abs(complex(r[0], r[1]) - ref) <= 1e-14 * np.linalg.norm(av) * np.linalg.norm(bv)


def test_dot_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    lib = q.lib()
    res = q.Field((2, 2, 2, 2))
    p = lib.qcdgpu_field_data(res.h)
    assert lib.qcdgpu_dot_noalloc(p, p, MAX_N + 1, p, None) == 1
    assert b"maximum" in lib.qcdgpu_last_error()


ALLOC_CHECK = """
import ctypes as C
import qcd_gb300 as q
lib = q.lib()
lib.qcdgpu_scratch_bytes.restype = C.c_int64
a, b, res = q.Field((8, 4, 4, 4)).gaussian(1), q.Field((8, 4, 4, 4)).gaussian(2), q.Field((2, 2, 2, 2))
pa, pb, pr = (lib.qcdgpu_field_data(f.h) for f in (a, b, res))
q.sync()
before = lib.qcdgpu_scratch_bytes()
for _ in range(3):
    assert lib.qcdgpu_dot_noalloc(pa, pb, a.nbytes // 16, pr, None) == 0
q.sync()
after = lib.qcdgpu_scratch_bytes()
a.dot(b)  # the regular dot allocates the reduction scratch on first use
print(before, after, lib.qcdgpu_scratch_bytes())
"""


def test_dot_noalloc_allocates_nothing(gpu):
    """in a fresh process, before any other reduction: three calls leave the
    library's lazily allocated reduction scratch unallocated, which the
    regular dot then allocates"""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", ALLOC_CHECK], cwd=root, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    before, after, regular = (int(x) for x in out.stdout.split()[-3:])
    assert before == 0 and after == 0
    assert regular > 0

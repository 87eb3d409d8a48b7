"""kz_exact.h on the CPU: the integer round-to-nearest-even int64 -> binary32 conversion the kernels use
(compiled from the same header) equals the IEEE conversion on edge cases and on random values."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER_DIR = os.path.join(ROOT, "kazan_gb300", "csrc", "raster")


@pytest.fixture(scope="module")
def conv(tmp_path_factory):
    d = tmp_path_factory.mktemp("exact")
    src = d / "t.c"
    src.write_text('#include "kz_exact.h"\n'
                   "void conv(const long long* v, unsigned* out, long n) {\n"
                   "  for (long i = 0; i < n; i++) out[i] = kz_i64_to_f32_bits((int64_t)v[i]);\n}\n")
    lib = d / "libt.so"
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-I", HEADER_DIR, str(src), "-o", str(lib)], check=True)
    L = ctypes.CDLL(str(lib))
    L.conv.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]

    def f(values):
        v = np.ascontiguousarray(values, dtype=np.int64)
        out = np.empty(len(v), dtype=np.uint32)
        L.conv(v.ctypes.data, out.ctypes.data, len(v))
        return out
    return f


def test_int64_to_float32_matches_ieee(conv):
    rng = np.random.default_rng(3)
    edges = [0, 1, -1, 2**24 - 1, 2**24, 2**24 + 1, 2**24 + 3, 2**25 + 2, 2**31 - 1, -2**31, 2**62 + 2**38,
             2**63 - 1, -2**63 + 1, -(2**40) - 2**16]
    vals = [np.array(edges, dtype=np.int64)]
    for bits in range(1, 63):
        vals.append(rng.integers(-(2**bits), 2**bits, 20000, dtype=np.int64))
    # exact halfway cases between neighbouring floats above 2^24
    for e in range(25, 62):
        base = rng.integers(2**23, 2**24, 2000, dtype=np.int64) << (e - 23)
        vals.append(base + (1 << (e - 24)))
        vals.append(-(base + (1 << (e - 24))))
    v = np.concatenate(vals)
    assert np.array_equal(conv(v), v.astype(np.float32).view(np.uint32))

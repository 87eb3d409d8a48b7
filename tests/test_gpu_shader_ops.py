"""GPU checks of the SPIR-V translator's arithmetic: every operation below runs in a fragment shader over 256
flat inputs and its 32-bit results come back bit for bit (tests/shader_ops.py).  Operations built from
correctly rounded single operations are compared bit for bit with a restatement of the same sequence (fma
rounded once, through exact rationals; a NaN matches any NaN, payloads being unspecified).  The
transcendental ones, which use the hardware exp2 / log2 / sin / cos approximations, are compared with numpy
in float64 within the tolerance given beside each."""
from fractions import Fraction

import numpy as np
import pytest

from kazan_gb300 import render, spirv_asm as sa

import shader_ops as so
from shader_ops import f32, fma

N = 256


def _rand(rng, lo, hi, n=N):
    return rng.uniform(lo, hi, n).astype(np.float32)


def _bits_f(rng, n=N):
    """random 32-bit patterns that are finite floats (flat inputs are copied, never computed on)"""
    u = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    u[(u >> 23 & 0xFF) == 0xFF] &= 0xBFFFFFFF
    return u.view(np.float32)


def _const32(dec):
    """a decimal float literal as the C++ compiler rounds it: once, to the nearest float32"""
    return so.round_f32(Fraction(dec))


def _i32(v):
    return int(np.float32(v).view(np.int32))


def _u32(v):
    return int(np.float32(v).view(np.uint32))


# op name -> (inputs(rng) float32 [N, 4], body(ctx) -> (id, kind), expected(x, y, z, w) -> value, tolerance)
# tolerance None: bit-exact; (atol, rtol): |gpu - ref| <= atol + rtol |ref| (ref in float64)
OPS = {}


def op(name, tol=None):
    def deco(f):
        OPS[name] = (f, tol)
        return f
    return deco


def _cols(*cols):
    return np.stack([np.asarray(c, dtype=np.float32) for c in cols], axis=1)


@op("fmod")
def _fmod(rng):
    y = _rand(rng, 0.5, 10) * rng.choice([-1, 1], N).astype(np.float32)
    return (_cols(_rand(rng, -100, 100), y, np.zeros(N), np.zeros(N)),
            lambda c: (c.m.res(so.OpFMod, c.f32, c.x, c.y), "f32"),
            lambda x, y, z, w: fma(-f32(y), np.floor(f32(x) / f32(y)), x))


@op("frem")
def _frem(rng):
    y = _rand(rng, 0.5, 10) * rng.choice([-1, 1], N).astype(np.float32)
    return (_cols(_rand(rng, -100, 100), y, np.zeros(N), np.zeros(N)),
            lambda c: (c.m.res(so.OpFRem, c.f32, c.x, c.y), "f32"),
            lambda x, y, z, w: fma(-f32(y), np.trunc(f32(x) / f32(y)), x))


@op("fsign")
def _fsign(rng):
    x = _rand(rng, -5, 5)
    x[::7] = 0.0
    x[1::11] = -0.0
    return (_cols(x, x, x, x), lambda c: (c.ext(c.f32, "FSign", c.x), "f32"),
            lambda x, y, z, w: f32(1.0) if x > 0 else (f32(-1.0) if x < 0 else f32(0.0)))


@op("radians")
def _radians(rng):
    x = _rand(rng, -720, 720)
    return (_cols(x, x, x, x), lambda c: (c.ext(c.f32, "Radians", c.x), "f32"),
            lambda x, y, z, w: f32(x) * _const32("0.0174532925"))


@op("degrees")
def _degrees(rng):
    x = _rand(rng, -7, 7)
    return (_cols(x, x, x, x), lambda c: (c.ext(c.f32, "Degrees", c.x), "f32"),
            lambda x, y, z, w: f32(x) * _const32("57.2957795"))


@op("smoothstep")
def _smoothstep(rng):
    def ref(x, y, z, w):
        t = (f32(z) - f32(x)) / (f32(y) - f32(x))
        t = min(max(t, f32(0)), f32(1))
        return (t * t) * fma(-2.0, t, 3.0)
    return (_cols(_rand(rng, -1, 0), _rand(rng, 1, 2), _rand(rng, -2, 3), np.zeros(N)),
            lambda c: (c.ext(c.f32, "SmoothStep", c.x, c.y, c.z), "f32"), ref)


@op("reflect")
def _reflect(rng):
    def body(c):
        r = c.ext(c.v2, "Reflect", c.vec2(c.x, c.y), c.vec2(c.z, c.w))
        return c.m.res(sa.OpCompositeExtract, c.f32, r, 0), "f32"

    def ref(x, y, z, w):
        d = fma(w, y, f32(z) * f32(x))
        return fma(-(f32(2.0) * d), z, x)
    return _cols(*[_rand(rng, -3, 3) for _ in range(4)]), body, ref


@op("faceforward")
def _faceforward(rng):
    def body(c):
        r = c.ext(c.v2, "FaceForward", c.vec2(c.x, c.y), c.vec2(c.z, c.w), c.vec2(c.y, c.x))
        return c.m.res(sa.OpCompositeExtract, c.f32, r, 1), "f32"

    def ref(x, y, z, w):
        d = fma(x, w, f32(y) * f32(z))
        return f32(y) if d < 0 else -f32(y)
    return _cols(*[_rand(rng, -3, 3) for _ in range(4)]), body, ref


@op("refract")
def _refract(rng):
    eta = f32(0.66)

    def body(c):
        r = c.ext(c.v2, "Refract", c.vec2(c.x, c.y), c.vec2(c.z, c.w), c.m.cf(0.66))
        return c.m.res(sa.OpCompositeExtract, c.f32, r, 0), "f32"

    def ref(x, y, z, w):
        d = fma(w, y, f32(z) * f32(x))
        k = f32(1.0) - (eta * eta) * fma(-d, d, 1.0)
        if k < 0:
            return f32(0.0)
        f = fma(eta, d, np.sqrt(k))
        return fma(eta, x, -(f * f32(z)))
    return _cols(*[_rand(rng, -1, 1) for _ in range(4)]), body, ref


@op("ldexp")
def _ldexp(rng):
    e = rng.integers(-20, 21, N).astype(np.float32)
    return (_cols(_rand(rng, -100, 100), e, np.zeros(N), np.zeros(N)),
            lambda c: (c.ext(c.f32, "Ldexp", c.x, c.to_int(c.y)), "f32"),
            lambda x, y, z, w: f32(np.ldexp(np.float64(x), int(y))))


def _mat2(c):
    m2 = c.m.mat(c.v2, 2)
    return m2, c.m.res(sa.OpCompositeConstruct, m2, c.vec2(c.x, c.y), c.vec2(c.z, c.w))


@op("determinant2")
def _det2(rng):
    def body(c):
        _, mat = _mat2(c)
        return c.ext(c.f32, "Determinant", mat), "f32"
    return (_cols(*[_rand(rng, -4, 4) for _ in range(4)]), body,
            lambda x, y, z, w: fma(x, w, -(f32(z) * f32(y))))


@op("inverse2")
def _inv2(rng):
    def body(c):
        m2, mat = _mat2(c)
        inv = c.ext(m2, "MatrixInverse", mat)
        return c.m.res(sa.OpCompositeExtract, c.f32, inv, 0, 0), "f32"

    def ref(x, y, z, w):
        det = fma(z, -f32(y), f32(x) * f32(w))
        return f32(w) * (f32(1.0) / det)
    return _cols(*[_rand(rng, 0.5, 4) for _ in range(4)]), body, ref


@op("packUnorm4x8")
def _pack_unorm(rng):
    def ref(*v):
        r = 0
        for k, c in enumerate(v):
            q = int(np.rint(min(max(f32(c), f32(0)), f32(1)) * f32(255.0)))
            r |= (q & 0xFF) << (8 * k)
        return r
    return (_cols(*[_rand(rng, -0.2, 1.2) for _ in range(4)]),
            lambda c: (c.ext(c.u32, "PackUnorm4x8", c.a), "u32"), ref)


@op("packSnorm4x8")
def _pack_snorm(rng):
    def ref(*v):
        r = 0
        for k, c in enumerate(v):
            q = int(np.rint(min(max(f32(c), f32(-1)), f32(1)) * f32(127.0)))
            r |= (q & 0xFF) << (8 * k)
        return r
    return (_cols(*[_rand(rng, -1.2, 1.2) for _ in range(4)]),
            lambda c: (c.ext(c.u32, "PackSnorm4x8", c.a), "u32"), ref)


@op("unpackUnorm4x8")
def _unpack_unorm(rng):
    def body(c):
        v = c.ext(c.v4, "UnpackUnorm4x8", c.bits(c.x))
        return c.m.res(sa.OpCompositeExtract, c.f32, v, 1), "f32"
    return (_cols(_bits_f(rng), np.zeros(N), np.zeros(N), np.zeros(N)), body,
            lambda x, y, z, w: f32((_u32(x) >> 8) & 0xFF) / f32(255.0))


@op("unpackSnorm4x8")
def _unpack_snorm(rng):
    def body(c):
        v = c.ext(c.v4, "UnpackSnorm4x8", c.bits(c.x))
        return c.m.res(sa.OpCompositeExtract, c.f32, v, 2), "f32"

    def ref(x, y, z, w):
        b = (_u32(x) >> 16) & 0xFF
        b = b - 256 if b >= 128 else b
        return max(f32(b) / f32(127.0), f32(-1.0))
    return _cols(_bits_f(rng), np.zeros(N), np.zeros(N), np.zeros(N)), body, ref


@op("packHalf2x16")
def _pack_half(rng):
    x = _rand(rng, -70000, 70000)
    x[::5] = _rand(rng, -1e-5, 1e-5, len(x[::5]))
    return (_cols(x, _rand(rng, -2, 2), np.zeros(N), np.zeros(N)),
            lambda c: (c.ext(c.u32, "PackHalf2x16", c.vec2(c.x, c.y)), "u32"),
            lambda x, y, z, w: int(np.float16(f32(x)).view(np.uint16)) | (int(np.float16(f32(y)).view(np.uint16)) << 16))


@op("unpackHalf2x16")
def _unpack_half(rng):
    def body(c):
        v = c.ext(c.v2, "UnpackHalf2x16", c.bits(c.x))
        return c.m.res(sa.OpCompositeExtract, c.f32, v, 1), "f32"
    return (_cols(_bits_f(rng), np.zeros(N), np.zeros(N), np.zeros(N)), body,
            lambda x, y, z, w: f32(np.uint16(_u32(x) >> 16).view(np.float16)))


@op("findILsb")
def _find_ilsb(rng):
    x = _bits_f(rng)
    x[::9] = 0.0
    return (_cols(x, x, x, x), lambda c: (c.ext(c.i32, "FindILsb", c.bits(c.x)), "i32"),
            lambda x, y, z, w: -1 if _u32(x) == 0 else (_u32(x) & -_u32(x)).bit_length() - 1)


@op("findUMsb")
def _find_umsb(rng):
    x = _bits_f(rng)
    x[::9] = 0.0
    return (_cols(x, x, x, x), lambda c: (c.ext(c.i32, "FindUMsb", c.bits(c.x)), "i32"),
            lambda x, y, z, w: _u32(x).bit_length() - 1)


@op("findSMsb")
def _find_smsb(rng):
    x = _bits_f(rng)
    x[::9] = 0.0
    return (_cols(x, x, x, x), lambda c: (c.ext(c.i32, "FindSMsb", c.m.res(sa.OpBitcast, c.i32, c.x)), "i32"),
            lambda x, y, z, w: (~_i32(x) if _i32(x) < 0 else _i32(x)).bit_length() - 1)


@op("sabs_ssign")
def _sabs(rng):
    def body(c):
        i = c.m.res(sa.OpBitcast, c.i32, c.x)
        a = c.ext(c.i32, "SAbs", i)
        s = c.ext(c.i32, "SSign", i)
        return c.m.res(sa.OpIAdd, c.i32, a, c.m.res(sa.OpIMul, c.i32, s, c.m.ci(1000))), "i32"
    x = _bits_f(rng)
    x[::9] = 0.0

    def ref(x, y, z, w):
        i = _i32(x)
        return ((abs(i) if i != -2 ** 31 else i) + 1000 * ((i > 0) - (i < 0))) & 0xFFFFFFFF
    return _cols(x, x, x, x), body, ref


@op("sclamp")
def _sclamp(rng):
    lo = rng.integers(-1000, 0, N)
    hi = lo + rng.integers(0, 2000, N)
    v = rng.integers(-3000, 3000, N)
    return (_cols(v, lo, hi, np.zeros(N)),
            lambda c: (c.ext(c.i32, "SClamp", c.to_int(c.x), c.to_int(c.y), c.to_int(c.z)), "i32"),
            lambda x, y, z, w: min(max(int(x), int(y)), int(z)))


@op("uclamp")
def _uclamp(rng):
    lo = rng.integers(0, 1000, N)
    hi = lo + rng.integers(0, 2000, N)
    v = rng.integers(0, 4000, N)

    def body(c):
        u = [c.m.res(sa.OpBitcast, c.u32, c.to_int(t)) for t in (c.x, c.y, c.z)]
        return c.ext(c.u32, "UClamp", *u), "u32"
    return _cols(v, lo, hi, np.zeros(N)), body, lambda x, y, z, w: min(max(int(x), int(y)), int(z))


@op("smod")
def _smod(rng):
    y = rng.integers(1, 50, N) * rng.choice([-1, 1], N)
    return (_cols(rng.integers(-1000, 1000, N), y, np.zeros(N), np.zeros(N)),
            lambda c: (c.m.res(so.OpSMod, c.i32, c.to_int(c.x), c.to_int(c.y)), "i32"),
            lambda x, y, z, w: int(x) % int(y))


@op("bitcount_reverse")
def _bitcount(rng):
    def body(c):
        u = c.bits(c.x)
        cnt = c.m.res(so.OpBitCount, c.u32, u)
        rev = c.m.res(so.OpBitReverse, c.u32, u)
        return c.m.res(sa.OpIAdd, c.u32, rev, cnt), "u32"

    def ref(x, y, z, w):
        u = _u32(x)
        return (int(format(u, "032b")[::-1], 2) + bin(u).count("1")) & 0xFFFFFFFF
    return _cols(_bits_f(rng), np.zeros(N), np.zeros(N), np.zeros(N)), body, ref


def _field_inputs(rng):
    off = rng.integers(0, 32, N)
    cnt = np.array([rng.integers(0, 33 - o) for o in off])
    return off, cnt


@op("bitfieldUExtract")
def _bfu(rng):
    off, cnt = _field_inputs(rng)
    return (_cols(_bits_f(rng), off, cnt, np.zeros(N)),
            lambda c: (c.m.res(so.OpBitFieldUExtract, c.u32, c.bits(c.x), c.to_int(c.y), c.to_int(c.z)), "u32"),
            lambda x, y, z, w: (_u32(x) >> int(y)) & ((1 << int(z)) - 1))


@op("bitfieldSExtract")
def _bfs(rng):
    off, cnt = _field_inputs(rng)

    def ref(x, y, z, w):
        cnt = int(z)
        if cnt == 0:
            return 0
        v = (_u32(x) >> int(y)) & ((1 << cnt) - 1)
        if v >> (cnt - 1):
            v -= 1 << cnt
        return v & 0xFFFFFFFF
    return (_cols(_bits_f(rng), off, cnt, np.zeros(N)),
            lambda c: (c.m.res(so.OpBitFieldSExtract, c.i32, c.m.res(sa.OpBitcast, c.i32, c.x), c.to_int(c.y),
                                c.to_int(c.z)), "i32"), ref)


@op("bitfieldInsert")
def _bfi(rng):
    off, cnt = _field_inputs(rng)

    def ref(x, y, z, w):
        mask = (((1 << int(w)) - 1) << int(z)) & 0xFFFFFFFF
        return (_u32(x) & ~mask & 0xFFFFFFFF) | ((_u32(y) << int(z)) & mask)
    return (_cols(_bits_f(rng), _bits_f(rng), off, cnt),
            lambda c: (c.m.res(so.OpBitFieldInsert, c.u32, c.bits(c.x), c.bits(c.y), c.to_int(c.z), c.to_int(c.w)),
                       "u32"), ref)


@op("any_all_isinf")
def _any_all(rng):
    def body(c):
        bvec = c.m.vec(c.m.bool(), 4)
        gt = c.m.res(sa.OpFOrdGreaterThan, bvec, c.a, c.m.cvec([0, 0, 0, 0]))
        one, zero = c.m.ci(1, 0), c.m.ci(0, 0)
        r_any = c.m.res(sa.OpSelect, c.u32, c.m.res(so.OpAny, c.m.bool(), gt), one, zero)
        r_all = c.m.res(sa.OpSelect, c.u32, c.m.res(so.OpAll, c.m.bool(), gt), c.m.ci(2, 0), zero)
        r_inf = c.m.res(sa.OpSelect, c.u32, c.m.res(so.OpIsInf, c.m.bool(), c.x), c.m.ci(4, 0), zero)
        return c.m.res(sa.OpIAdd, c.u32, c.m.res(sa.OpIAdd, c.u32, r_any, r_all), r_inf), "u32"
    v = rng.choice([-1.0, 1.0], (N, 4)).astype(np.float32)
    v[::13, 0] = np.inf
    v[5::13, 0] = -np.inf

    def ref(x, y, z, w):
        g = [t > 0 for t in (x, y, z, w)]
        return int(any(g)) + 2 * int(all(g)) + 4 * int(np.isinf(x))
    return v, body, ref


def _approx(name, lo, hi, fn, tol, nargs=1, lo2=None, hi2=None):
    @op(name, tol)
    def _f(rng):
        ys = _rand(rng, lo2, hi2) if nargs == 2 else np.zeros(N)
        body = (lambda c: (c.ext(c.f32, name.capitalize() if name != "atan2" else "Atan2", c.x, c.y), "f32")) \
            if nargs == 2 else (lambda c: (c.ext(c.f32, name.capitalize(), c.x), "f32"))
        return _cols(_rand(rng, lo, hi), ys, np.zeros(N), np.zeros(N)), body, fn
    return _f


_approx("exp", -10, 10, lambda x, y, z, w: np.exp(np.float64(x)), (2e-6, 4e-6))
_approx("log", 1e-3, 1e3, lambda x, y, z, w: np.log(np.float64(x)), (2e-6, 4e-6))
_approx("tan", -1.2, 1.2, lambda x, y, z, w: np.tan(np.float64(x)), (2e-6, 6e-6))
_approx("sinh", -5, 5, lambda x, y, z, w: np.sinh(np.float64(x)), (2e-6, 4e-6))
_approx("cosh", -5, 5, lambda x, y, z, w: np.cosh(np.float64(x)), (2e-6, 4e-6))
_approx("tanh", -3, 3, lambda x, y, z, w: np.tanh(np.float64(x)), (2e-6, 4e-6))
_approx("asinh", -20, 20, lambda x, y, z, w: np.arcsinh(np.float64(x)), (2e-6, 4e-6))
_approx("acosh", 1.001, 30, lambda x, y, z, w: np.arccosh(np.float64(x)), (1e-5, 4e-6))
_approx("atanh", -0.9, 0.9, lambda x, y, z, w: np.arctanh(np.float64(x)), (2e-6, 4e-6))
_approx("atan", -50, 50, lambda x, y, z, w: np.arctan(np.float64(x)), (2e-6, 4e-6))
_approx("asin", -0.99, 0.99, lambda x, y, z, w: np.arcsin(np.float64(x)), (2e-6, 4e-6))
_approx("acos", -0.99, 0.99, lambda x, y, z, w: np.arccos(np.float64(x)), (2e-6, 4e-6))
_approx("atan2", -5, 5, lambda x, y, z, w: np.arctan2(np.float64(x), np.float64(y)), (2e-6, 4e-6), 2, -5, 5)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(OPS))
def test_shader_op(renderer, name):
    make, tol = OPS[name]
    rng = np.random.default_rng(sum(map(ord, name)))
    inputs, body, ref = make(rng)
    scene = so.cell_scene(inputs, so.op_fs(body))
    run = render.SceneRun(renderer, scene, mode="batched", tile=16)
    run.submit()
    color, _ = run.read()
    renderer.free_command_buffer(run.cb)
    got = so.read_bits(color, len(inputs))
    bad = []
    for i, v in enumerate(inputs):
        want = ref(*[np.float32(t) for t in v])
        if tol is None:
            is_f = isinstance(want, (np.floating, float))
            if is_f and np.isnan(want):  # NaN payloads are not specified: any NaN
                if not np.isnan(np.uint32(got[i]).view(np.float32)):
                    bad.append((i, v.tolist(), hex(int(got[i])), "NaN"))
                continue
            wb = so.bits(want) if is_f else int(want) & 0xFFFFFFFF
            if int(got[i]) != wb:
                bad.append((i, v.tolist(), hex(int(got[i])), hex(wb)))
        else:
            g = float(np.uint32(got[i]).view(np.float32))
            if not abs(g - float(want)) <= tol[0] + tol[1] * abs(float(want)):
                bad.append((i, v.tolist(), g, float(want)))
    assert not bad, "%s: %d of %d differ, first %s" % (name, len(bad), len(inputs), bad[:3])

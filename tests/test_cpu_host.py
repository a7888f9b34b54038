"""CPU tests: index maps, host logic, the device integral math compiled as
host C++ against the oracle, and the C-ABI library's exported symbols and
argument checks (no compute call needs a GPU here)."""
from __future__ import annotations

import ctypes as C
import itertools
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT


# ---------------------------------------------------------------- index maps
def _py_index(ne, np_, ip, jp, *e):
    acc = (ip - 1)
    acc = (jp - 1) + np_ * acc
    for x in e:
        acc = (x - 1) + ne * acc
    return 1 + acc


@pytest.mark.parametrize("ne,np_", [(1, 1), (2, 3), (3, 2), (4, 1)])
def test_index_maps_are_the_loop_order(orc, ne, np_):
    """index_GAM_2PK/3PK/4PK2 (pack_GAM.f:72-239) enumerate 1..N in the
    reference's loop order (ip, jp, ie1, je1, ... last ket fastest)."""
    L = orc.lib()
    for k, fn in ((2, L.orc_index_gam_2pk), (3, L.orc_index_gam_3pk), (4, L.orc_index_gam_4pk2)):
        if ne ** (2 * k) * np_ ** 2 > 70000:
            continue
        t = 0
        for ip, jp in itertools.product(range(1, np_ + 1), repeat=2):
            for e in itertools.product(range(1, ne + 1), repeat=2 * k):
                t += 1
                v = fn(ne, np_, ip, jp, *e)
                assert v == t == _py_index(ne, np_, ip, jp, *e)


def test_index_4pk2_is_int64(orc):
    L = orc.lib()
    big = L.orc_index_gam_4pk2(40, 20, 20, 20, *([40] * 8))
    assert big == 40 ** 8 * 20 ** 2 > 2 ** 62 // 2 ** 20


def test_loop_size_partition(orc):
    """gam_2_OMP.f:1080-1095 loop_size splits [L1,L2] into contiguous,
    covering, near-equal chunks (the multi-GPU range split)."""
    L = orc.lib()
    for n, parts in ((10, 3), (7, 7), (5, 8), (1000003, 16)):
        got = []
        for r in range(parts):
            a, b = np.zeros(1, np.int64), np.zeros(1, np.int64)
            L.orc_loop_size(1, n, parts, r, orc.ptr(a), orc.ptr(b))
            got.append((int(a[0]), int(b[0])))
        flat = [x for a, b in got for x in range(a, b + 1)]
        assert flat == list(range(1, n + 1))
        sizes = [b - a + 1 for a, b in got]
        assert max(sizes) - min(sizes) <= 1


# ---------------------------------------------------------------- basis logic
def test_make_kpe_and_normalisation(orc, golden_xchf):
    from neoxc import basis
    s = basis.parse_inp(golden_xchf["inp"])
    assert list(s.KPESTR) == [1, 4, 5, 8, 9, 12] and list(s.KPEEND) == [3, 4, 7, 8, 11, 12]
    # normalised coefficients printed by the reference (XCHF.log, 6 decimals)
    np.testing.assert_allclose(s.AGEBFCC[:4], [0.441353, 0.693497, 0.664184, 0.287167], atol=5e-7)
    np.testing.assert_allclose(s.AGNBFCC, [2.077622], atol=5e-7)
    # Python restatement == oracle restatement of ELCNORM3 / NUCNORM
    L = orc.lib()
    raw = basis.parse_inp.__globals__["_card_lines"](golden_xchf["inp"], "EBASIS", s.npebf)
    coef = np.array([float(r[6]) for r in raw])
    L.orc_elcnorm3(s.npebf, s.nebf, orc.ptr(s.AMPEB2C_f), orc.ptr(coef), orc.ptr(s.ELCEX_f),
                   orc.ptr(s.ELCAM_f), orc.ptr(s.ELCBFC_f))
    np.testing.assert_allclose(coef, s.AGEBFCC, rtol=1e-13)
    kps, kpe = np.zeros(s.nebf, np.int64), np.zeros(s.nebf, np.int64)
    L.orc_make_kpe(s.nebf, s.npebf, orc.ptr(s.AMPEB2C_f), orc.ptr(kps), orc.ptr(kpe))
    assert np.array_equal(kps, s.KPESTR) and np.array_equal(kpe, s.KPEEND)


def test_mo_reader_and_density(golden_xchf):
    from neoxc import basis
    vec = basis.read_mo_file(golden_xchf["guessCE"], 6)
    assert vec[0, 0] == pytest.approx(0.402716176) and vec[5, 0] == pytest.approx(-1.68233830e-3)
    D = basis.density(vec, 2, 2.0)
    assert np.allclose(D, D.T)
    assert D[0, 0] == pytest.approx(2 * (vec[0, 0] ** 2 + vec[0, 1] ** 2))


def test_synthetic_is_seeded():
    from neoxc import basis
    a = basis.synthetic(seed=3, nebf=5, npbf=3)
    b = basis.synthetic(seed=3, nebf=5, npbf=3)
    assert np.array_equal(a.ELCEX, b.ELCEX) and np.array_equal(a.cat, b.cat)
    assert a.npebf == 15 and a.ng2 == 5 ** 4 * 9


# ------------------------------------- device integral math, host-compiled
@pytest.fixture(scope="module")
def hostcheck():
    src = os.path.join(ROOT, "tests", "hostcheck", "md_host_check.cpp")
    out = os.path.join(tempfile.mkdtemp(prefix="neoxc_hc_"), "libhc.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", src, "-o", out], check=True)
    L = C.CDLL(out)
    return L


def test_md_math_matches_oracle(orc, hostcheck):
    """The factorised MD evaluation the kernels run (md_math.cuh) against the
    oracle's restatement of the reference loops, random s/p/d primitives."""
    O, L, H = orc, orc.lib(), hostcheck
    P = C.POINTER(O.Prim)
    d = C.c_double
    H.hc_g3.restype = d
    H.hc_g3.argtypes = [C.c_int, P, P, C.c_void_p, C.c_void_p, d]
    H.hc_g4.restype = d
    H.hc_g4.argtypes = [C.c_int, P, P, d, d]
    for f in ("hc_g2_xggs", "hc_g2_xggvee"):
        getattr(H, f).restype = d
        getattr(H, f).argtypes = [P, P, P, P, d, d]
    H.hc_g2_xggvec.restype = d
    H.hc_g2_xggvec.argtypes = [P, P, P, P, d, d, C.c_void_p]
    H.hc_pgike1.restype = d
    H.hc_pgike1.argtypes = [P, P, P, P, d, d, d]
    H.hc_gfvee.restype = d
    H.hc_gfvee.argtypes = [P, P, P, P]
    H.hc_gfke.restype = d
    H.hc_gfke.argtypes = [P, P, d]
    H.hc_gfvec.restype = d
    H.hc_gfvec.argtypes = [P, P, C.c_void_p]
    rng = np.random.default_rng(1)
    AMS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (1, 1, 0), (0, 2, 0),
           (1, 0, 1), (0, 1, 1), (0, 0, 2)]

    def rp():
        l = AMS[rng.integers(0, len(AMS))]
        return O.prim(*l, float(np.exp(rng.uniform(np.log(0.1), np.log(20)))),
                      *rng.uniform(-1.5, 1.5, 3))

    def check(a, b, what):
        # relative on significant values, absolute floor for cancelled ones
        assert abs(a - b) <= 1e-10 * abs(b) + 1e-14, (what, a, b)

    def sp():   # an s primitive (the s-shell fast paths)
        return O.prim(0, 0, 0, float(np.exp(rng.uniform(np.log(0.1), np.log(20)))),
                      *rng.uniform(-1.5, 1.5, 3))

    for trial in range(35):
        if trial < 25:
            A = O.prims([rp() for _ in range(4)])
            B = O.prims([rp() for _ in range(4)])
        else:
            A = O.prims([sp() for _ in range(4)])
            B = O.prims([sp() for _ in range(4)])
        g = np.zeros(6)
        for k in rng.choice(6, size=2, replace=False):
            g[k] = float(np.exp(rng.uniform(np.log(0.5), np.log(20))))
        Cm = rng.uniform(-1.5, 1.5, 3)
        A3, B3 = O.prims([A[0], A[1], A[2]]), O.prims([B[0], B[1], B[2]])
        check(H.hc_g3(0, A3, B3, O.ptr(g), O.ptr(Cm), 1.0), L.orc_g3_xggs(A3, B3, O.ptr(g)), "xggs")
        gk = g.copy()
        gk[3] = 0.0
        check(H.hc_g3(1, A3, B3, O.ptr(gk), O.ptr(Cm), 1.0), L.orc_g3_ke(A3, B3, O.ptr(gk), 1.0), "ke")
        check(H.hc_g3(2, A3, B3, O.ptr(g), O.ptr(Cm), 1.0),
              L.orc_g3_xgvxcg(A3, B3, O.ptr(g), O.ptr(Cm)), "vxc")
        check(H.hc_g3(3, A3, B3, O.ptr(g), O.ptr(Cm), 1.0), L.orc_g3_xgveeg(A3, B3, O.ptr(g)), "vee")
        g1, g2 = g[g > 0][0], g[g > 0][1]
        if trial < 10 or trial >= 25:
            check(H.hc_g4(0, A, B, g1, g2), L.orc_g4_xgveeg(A, B, g1, g2), "g4vee")
            check(H.hc_g4(1, A, B, g1, g2), L.orc_g4_xgvepg(A, B, g1, g2), "g4vep")
        r = [C.byref(A[0]), C.byref(A[1]), C.byref(B[0]), C.byref(B[1])]
        check(H.hc_g2_xggs(*r, g1, g2), L.orc_g2_xggs(*r, g1, g2), "g2")
        # gam_1 kernels (XC1_G2_MD.f, g2.f), with one geminal exponent zero as
        # in xcalc_GAM1_MD and with both set
        for ga, gb in ((g1, 0.0), (0.0, g1), (g1, g2)):
            check(H.hc_g2_xggvec(*r, ga, gb, O.ptr(Cm)),
                  L.orc_g2_xggvec(*r, ga, gb, O.ptr(Cm)), "g2vec")
            check(H.hc_g2_xggvee(*r, ga, gb), L.orc_g2_xggvee(*r, ga, gb), "g2vee")
            check(H.hc_pgike1(*r, ga, gb, 1836.0), L.orc_pgike1(*r, ga, gb, 1836.0, None),
                  "pgike1")
        check(H.hc_gfvee(*r), L.orc_gfvee(*r), "gfvee")
        check(H.hc_gfke(r[0], r[2], 1.0), L.orc_gfke(r[0], r[2], 1.0), "gfke")
        check(H.hc_gfvec(r[0], r[2], O.ptr(Cm)), L.orc_gfvec(r[0], r[2], O.ptr(Cm)), "gfvec")


def test_boys_function_matches_xgammaf(orc, hostcheck):
    """The kernels' FP64 Boys function (pretabulated Taylor expansion for
    T <= 20, XGAMMAF's asymptotic branch above) against the oracle's
    restatement of XGAMMAF (common.f:317-348), every order the kernels use.
    The table is exact to ~1e-15; XGAMMAF's series stops at a 1e-12 term,
    which leaves up to ~2.4e-12 relative in its values for T <= 20.  Above
    T = 20 both take XGAMMAF's asymptotic branch."""
    L, H = orc.lib(), hostcheck
    H.hc_boys.restype = C.c_double
    H.hc_boys.argtypes = [C.c_int, C.c_double]
    rng = np.random.default_rng(5)
    Ts = np.concatenate([[0.0, 1e-14, 1e-6, 0.03125, 19.97, 20.0, 20.0001, 35.0, 300.0],
                         rng.uniform(0, 22, 400), np.exp(rng.uniform(-20, 3, 100))])
    F = np.zeros(17)
    worst = 0.0
    for T in Ts:
        L.orc_xgammaf(orc.ptr(F), float(T), 16)
        for m in range(17):
            got = H.hc_boys(m, float(T))
            worst = max(worst, abs(got - F[m]) / F[m])
    assert worst < 5e-12, worst


def test_integer_narrowing_to_fp32(hostcheck):
    """tc::narrow_f64 (the tensor-core path's FP64 -> FP32 conversion on the
    integer pipes): significand truncated toward zero (|f| <= |v|, relative
    error below 2^-23, the FP32 rounding of v within one unit in the last
    place), signed zero below the FP32 normal range, infinity above it, NaN
    kept."""
    H = hostcheck
    H.hc_narrow.restype = C.c_float
    H.hc_narrow.argtypes = [C.c_double]
    rng = np.random.default_rng(12)
    vals = np.concatenate([rng.standard_normal(2000) * np.exp(rng.uniform(-80, 80, 2000)),
                           [1.0, -1.0, 3.0, 1.0 / 3.0, 2.0 ** -126, -(2.0 ** -126) * 1.5,
                            3.4e38, -3.4e38]])
    for v in vals:
        f = float(H.hc_narrow(float(v)))
        assert abs(f) <= abs(v) and np.sign(f) == np.sign(v), v
        assert abs(f - v) < 2.0 ** -23 * abs(v), v
        assert abs(f - float(np.float32(v))) <= float(np.spacing(np.float32(abs(v)))), v
    for v, want in ((0.0, 0.0), (1e-40, 0.0), (-1e-300, -0.0), (5e-324, 0.0)):
        f = float(H.hc_narrow(v))
        assert f == 0.0 and np.signbit(f) == np.signbit(want), v
    assert float(H.hc_narrow(1e39)) == float("inf")
    assert float(H.hc_narrow(-1e300)) == float("-inf")
    assert float(H.hc_narrow(float("inf"))) == float("inf")
    assert np.isnan(H.hc_narrow(float("nan")))


def test_fused_boys_seed_sum(orc, hostcheck):
    """boys_sum (the Boys recursion fused with the Horner sum of the seeds
    (-alpha)^m F_m(T) b_m) against XGAMMAF's restatement followed by the
    plain sum; and for an FP32 argument (grid offset formed in FP32, exact)
    bit-identical to the FP64 argument of the same value."""
    L, H = orc.lib(), hostcheck
    H.hc_boys_sum.restype = C.c_double
    H.hc_boys_sum.argtypes = [C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double), C.c_int]
    rng = np.random.default_rng(8)
    F = np.zeros(17)
    for trial in range(300):
        Lm = int(rng.integers(0, 17))
        T = float(np.float32(rng.choice([rng.uniform(0, 22), np.exp(rng.uniform(-12, 3))])))
        alpha = float(np.exp(rng.uniform(-2, 3)))
        b = rng.uniform(-1, 1, Lm + 1)
        pb = b.ctypes.data_as(C.POINTER(C.c_double))
        got = H.hc_boys_sum(Lm, T, alpha, pb, 0)
        L.orc_xgammaf(orc.ptr(F), T, 16)
        ref = sum((-alpha) ** m * F[m] * b[m] for m in range(Lm + 1))
        scale = sum(abs((-alpha) ** m * F[m] * b[m]) for m in range(Lm + 1))
        assert abs(got - ref) <= 1e-11 * scale, (Lm, T, alpha, got, ref)
        assert H.hc_boys_sum(Lm, T, alpha, pb, 1) == got, (Lm, T)


def test_composite_bra_form_matches_g4_integrals(orc, hostcheck):
    """The gam_3 builder evaluates G4_MD_xgVeeg / G4_MD_xgVepg as a Coulomb
    integral between a composite bra (three pair densities, both geminals
    integrated out) and the free electron's pair density, with the factorised
    Hermite-Coulomb sum (g3_fatbra.cuh).  FP64: the oracle's restatement of
    the reference's 12-deep loops (XC1_G4_MD.f) to 1e-10 relative; FP32 (the
    mixed path: FP32 tables, FP64 Boys function, seeds and sum): at the FP32
    level."""
    O, L, H = orc, orc.lib(), hostcheck
    P = C.POINTER(O.Prim)
    d = C.c_double
    for f in ("hc_fb", "hc32_fb"):
        getattr(H, f).restype = d
        getattr(H, f).argtypes = [C.c_int, P, P, d, d]
    rng = np.random.default_rng(21)
    AMS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (1, 1, 0), (0, 2, 0),
           (1, 0, 1), (0, 1, 1), (0, 0, 2)]

    def rp(lmax):
        ams = [a for a in AMS if sum(a) <= lmax]
        l = ams[rng.integers(0, len(ams))]
        return O.prim(*l, float(np.exp(rng.uniform(np.log(0.1), np.log(20)))),
                      *rng.uniform(-1.5, 1.5, 3))
    errs32 = []
    for trial in range(80):
        lm = (0, 1, 2)[trial % 3]
        A = O.prims([rp(lm) for _ in range(4)])
        B = O.prims([rp(lm) for _ in range(4)])
        g1, g2 = np.exp(rng.uniform(np.log(0.5), np.log(20), 2))
        for kind, ref in ((0, L.orc_g4_xgveeg(A, B, g1, g2)),
                          (1, L.orc_g4_xgvepg(A, B, g1, g2))):
            got = H.hc_fb(kind, A, B, g1, g2)
            assert abs(got - ref) <= 1e-10 * abs(ref) + 1e-14, (trial, kind, got, ref)
            g32 = H.hc32_fb(kind, A, B, g1, g2)
            if abs(ref) > 1e-12:
                errs32.append(abs(g32 - ref) / abs(ref))
    errs32 = np.array(errs32)
    assert errs32.max() < 2e-4 and np.median(errs32) < 3e-5, (errs32.max(), np.median(errs32))


def test_md32_instance_within_fp32_error(orc, hostcheck):
    """The mixed path's FP32 instance (md_math32.cuh: FP32 tables and
    recursions, FP64 Boys function and seeds) against the oracle's FP64
    four- and three-particle integrals on random s/p/d primitives: the
    relative error stays at the FP32 level (bound 2e-4 on significant
    values, 3e-5 on the median)."""
    O, L, H = orc, orc.lib(), hostcheck
    P = C.POINTER(O.Prim)
    d = C.c_double
    H.hc32_g4.restype = d
    H.hc32_g4.argtypes = [C.c_int, P, P, d, d]
    H.hc32_g3.restype = d
    H.hc32_g3.argtypes = [C.c_int, P, P, C.c_void_p, C.c_void_p, d]
    rng = np.random.default_rng(11)
    AMS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (1, 1, 0), (0, 2, 0),
           (1, 0, 1), (0, 1, 1), (0, 0, 2)]

    def rp():
        l = AMS[rng.integers(0, len(AMS))]
        return O.prim(*l, float(np.exp(rng.uniform(np.log(0.1), np.log(20)))),
                      *rng.uniform(-1.5, 1.5, 3))
    errs = []
    for trial in range(60):
        A = O.prims([rp() for _ in range(4)])
        B = O.prims([rp() for _ in range(4)])
        g1, g2 = np.exp(rng.uniform(np.log(0.5), np.log(20), 2))
        g = np.zeros(6)
        g[1], g[5] = g1, g2
        Cm = rng.uniform(-1.5, 1.5, 3)
        A3, B3 = O.prims([A[0], A[1], A[2]]), O.prims([B[0], B[1], B[2]])
        pairs = [(H.hc32_g4(0, A, B, g1, g2), L.orc_g4_xgveeg(A, B, g1, g2)),
                 (H.hc32_g4(1, A, B, g1, g2), L.orc_g4_xgvepg(A, B, g1, g2)),
                 (H.hc32_g3(3, A3, B3, O.ptr(g), O.ptr(Cm), 1.0),
                  L.orc_g3_xgveeg(A3, B3, O.ptr(g))),
                 (H.hc32_g3(2, A3, B3, O.ptr(g), O.ptr(Cm), 1.0),
                  L.orc_g3_xgvxcg(A3, B3, O.ptr(g), O.ptr(Cm)))]
        scale = max(abs(b) for _, b in pairs)
        for a, b in pairs:
            if abs(b) > 1e-6 * scale and abs(b) > 1e-30:
                errs.append(abs(a - b) / abs(b))
    errs = np.array(errs)
    assert errs.max() < 2e-4 and np.median(errs) < 3e-5, (errs.max(), np.median(errs))


# ------------------------------------------------------- C-ABI library (no GPU)
def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "neoxc.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b(?:int|int64_t|void|double|const char\*)\s+([a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    import neoxc
    L = neoxc.lib(build_if_missing=True)
    names = _header_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", neoxc.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(ln.split()[-1] for ln in out.splitlines() if ln.strip())
    assert set(names) <= exported


def _header_arg_counts():
    txt = open(os.path.join(ROOT, "include", "neoxc.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(?:int|int64_t|void|double|const char\*)\s+([a-z0-9_]+)\s*\(([^)]*)\)",
                         txt):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_ctypes_signatures_match_header():
    """Every ctypes prototype the Python mirror sets has the parameter count
    that include/neoxc.h declares (a mismatch would pass garbage over the
    C-ABI)."""
    import neoxc
    L = neoxc.lib(build_if_missing=True)
    want = _header_arg_counts()
    checked = 0
    for name, n in want.items():
        f = getattr(L, name)
        if f.argtypes is None:
            continue
        assert len(f.argtypes) == n, (name, len(f.argtypes), n)
        checked += 1
    assert checked >= 30


def test_mixed_threshold_argument_check():
    """neoxc_set_mixed_threshold is host-only: it accepts tau >= 0 (and
    infinity), refuses negative or NaN thresholds with NEOXC_ERR_ARG, and
    neoxc_get_mixed_threshold reads the value back."""
    import neoxc
    old = neoxc.get_mixed_threshold()
    assert old == 1e-5
    for bad in (-1.0, float("nan")):
        with pytest.raises(neoxc.NeoxcError):
            neoxc.set_mixed_threshold(bad)
    assert neoxc.get_mixed_threshold() == old
    neoxc.set_mixed_threshold(float("inf"))
    assert neoxc.get_mixed_threshold() == float("inf")
    neoxc.set_mixed_threshold(old)


def test_batch_job_struct_layout():
    """The Python mirror of neoxc_xchf_job has the C struct's size."""
    import ctypes
    import neoxc
    assert ctypes.sizeof(neoxc.XchfJob) == neoxc.lib(build_if_missing=True).neoxc_xchf_job_size()


def test_proton_scan_moves_only_the_proton_basis():
    from neoxc import basis
    s = basis.synthetic(seed=4, nat=2, nebf=3, nprim=1, npbf=2)
    scan = basis.proton_scan(s, 3, 0.5, seed=1)
    for t in scan:
        d = t.NUCBFC - s.NUCBFC
        assert np.all(np.abs(d) <= 0.5) and np.allclose(d, d[0])
        assert np.array_equal(t.ELCBFC, s.ELCBFC) and np.array_equal(t.cat, s.cat)


def test_admission_rule():
    """neoxc_admit, the memory-admission rule of the batch driver and the
    server: limit = 0.8 (free + in_use), lowered to the cap; a job above the
    limit is refused, one that fits starts, anything else waits; with
    nothing running a job never waits (no deadlock)."""
    import neoxc
    L = neoxc.lib(build_if_missing=True)
    S, W, R = neoxc.ADMIT_START, neoxc.ADMIT_WAIT, neoxc.ADMIT_REFUSE
    assert L.neoxc_admit(10, 100, 0, 0) == S
    assert L.neoxc_admit(90, 100, 0, 0) == R          # > 0.8 of everything
    assert L.neoxc_admit(30, 50, 50, 0) == S          # 50 + 30 <= 0.8 * 100
    assert L.neoxc_admit(40, 50, 50, 0) == W          # fits once a job ends
    assert L.neoxc_admit(10, 10 ** 12, 0, 5) == R     # above the cap
    assert L.neoxc_admit(10, 10 ** 12, 10, 15) == W   # cap shared with running jobs
    assert L.neoxc_admit(-1, 100, 0, 0) == R
    rng = np.random.default_rng(3)
    for need, free in rng.integers(0, 10 ** 11, size=(200, 2)):
        assert L.neoxc_admit(int(need), int(free), 0, 0) in (S, R)


def test_job_footprint_counts_the_tensors():
    """neoxc_xchf_job_bytes: the footprint neoxc_admit weighs holds at least
    the stored gam_2 and gam_3 tensors of the job's system."""
    import neoxc
    from neoxc import basis
    L = neoxc.lib(build_if_missing=True)
    s = basis.synthetic(seed=1, nebf=12, npbf=8)
    job = neoxc.XchfJob()
    keep = neoxc._fill_job(job, s, np.eye(12), None, 5)
    b = L.neoxc_xchf_job_bytes(C.byref(job), 0)
    assert b >= 8 * (2 * s.ng2 + s.ng3)
    assert keep["ne"] == 12


def test_argument_checks_need_no_gpu():
    """Size validation happens on the host before any device work, and a
    shape outside the supported range is an error, never a CPU fallback."""
    import neoxc
    L = neoxc.lib(build_if_missing=True)
    a = np.zeros(64)
    p = a.ctypes.data_as(C.c_void_p)
    # ng4 inconsistent with ne**8 np**2
    assert L.neoxc_gam4_dscf(1, 2, 1, 16, 16, 17, *([p] * 7)) == 1
    assert b"ng4" in L.neoxc_last_error()
    # Nchunks must be >= 1 (the reference's NG4CHK)
    assert L.neoxc_eg3ic1(0, 2, 1, 64, *([p] * 6)) == 1
    # map kind outside {0,2,3,4}
    assert L.neoxc_index_map(7, 2, 2, 4, p) == 1
    # host index maps are plain arithmetic
    assert L.neoxc_index_gam_2pk(3, 2, 2, 2, 3, 3, 3, 3) == 3 ** 4 * 4
    # an npbf beyond int range is refused before any narrowing (2^32 + 2
    # would otherwise wrap to 2), by both gam_4 device entry points
    for fn in (L.neoxc_dev_gam4_dscf, L.neoxc_dev_gam4_dscf_noalloc):
        assert fn(None, 12, 2 ** 32 + 2, *([p] * 7)) == 4
        assert b"np <=" in L.neoxc_last_error()
    # no device here: compute calls report a CUDA error instead of running
    if not L.neoxc_device_ok():
        assert b"CUDA" in L.neoxc_last_error() or b"device" in L.neoxc_last_error()

"""The reference's on-disk formats through the library's native readers and
writers (xchf1_independent/GAM_IO.f): FinalC*.dat / guessC*.inp MO files,
direct-access *.ufm integral files, ENUCRP.dat, and the by-reference
GAM_IO.f shims.  Host code only: these run without a GPU.

The pins are the reference's own files (tests/golden/xchf_example.json holds
examples/xchf/guessCE.inp and answer/FinalC{E,P}.dat verbatim): reading them
and writing them back must reproduce them byte for byte.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def F():
    import neoxc
    neoxc.lib(build_if_missing=True)
    from neoxc import formats
    return formats


@pytest.fixture
def in_tmp(tmp_path):
    old = os.getcwd()
    os.chdir(tmp_path)
    yield tmp_path
    os.chdir(old)


def _i64(v):
    return C.byref(C.c_int64(v))


@pytest.mark.parametrize("key,nbf", [("guessCE", 6), ("finalCE", 6), ("finalCP", 1)])
def test_mo_file_round_trip_is_byte_exact(F, golden_xchf, tmp_path, key, nbf):
    """PUSQLF's FORMAT(I2,I3,1P,5E15.8): read -> write gives the reference's
    file back unchanged."""
    src = tmp_path / "in.dat"
    src.write_text(golden_xchf[key])
    V = F.read_mos(src, nbf)
    out = tmp_path / "out.dat"
    F.write_mos(out, V)
    assert out.read_text() == golden_xchf[key]


def test_mo_read_matches_python_parser(F, golden_xchf, tmp_path):
    from neoxc import basis
    src = tmp_path / "g.inp"
    src.write_text(golden_xchf["guessCE"])
    assert np.array_equal(F.read_mos(src, 6), basis.read_mo_file(golden_xchf["guessCE"], 6))


def test_read_elec_density_is_the_guess_density(F, golden_xchf, xchf, tmp_path):
    """read_elec_density (GAM_IO.f:247-347): nelec/2 doubly occupied MOs."""
    src = tmp_path / "guessCE.inp"
    src.write_text(golden_xchf["guessCE"])
    DE = F.read_elec_density(src, 6, xchf["sys"].nelec)
    assert np.abs(DE - xchf["DE0"]).max() <= 1e-15
    # one particle: MO 1 alone, prefac 1
    V = F.read_mos(src, 6)
    assert np.allclose(F.read_elec_density(src, 6, 1), np.outer(V[:, 0], V[:, 0]),
                       rtol=0, atol=1e-15)


def test_mo_write_edge_values(F, tmp_path):
    """Ew.d with three-digit exponents drops the letter; -0, subnormals and
    rounding to a new power of ten keep the field at 15 columns."""
    v = np.array([1e-120, -0.0, 1e100, 123.456, -9.99999999999e-100, 5e-324, 9.9999999996,
                  -1.0, 0.0, 7.0])
    p = tmp_path / "e.dat"
    F.write_mos(p, v[:, None])
    lines = p.read_text().splitlines()
    assert lines == [
        " 1  1 1.00000000-120-0.00000000E+00 1.00000000+100 1.23456000E+02-1.00000000E-99",
        " 1  2 4.94065646-324 1.00000000E+01-1.00000000E+00 0.00000000E+00 7.00000000E+00",
    ]
    back = F.read_mos(p, 10, 1)[:, 0]
    assert np.allclose(back, [1e-120, 0, 1e100, 123.456, -1e-99, 4.94065646e-324, 10.0, -1,
                              0, 7], rtol=1e-15, atol=0)


def test_mo_read_fortran_input_forms(F, tmp_path):
    """Ew.d input: E/D exponents, an exponent without its letter, a field
    without a decimal point (8 implied decimals), and blank fields (0)."""
    fields = ["  1.5D+02", "   2.5-101", "  123456789", "", " -3.25e-1"]
    line = " 1  1" + "".join(f.rjust(15) for f in fields)
    p = tmp_path / "f.inp"
    p.write_text(line + "\n")
    got = F.read_mos(p, 5, 1)[:, 0]
    assert np.allclose(got, [150.0, 2.5e-101, 1.23456789, 0.0, -0.325], rtol=1e-15, atol=0)


def test_mo_read_rejects_bad_labels_and_short_files(F, golden_xchf, tmp_path):
    import neoxc
    txt = golden_xchf["finalCE"].splitlines()
    bad = tmp_path / "bad.dat"
    bad.write_text("\n".join([txt[0], " 9  2" + txt[1][5:]] + txt[2:]) + "\n")
    with pytest.raises(neoxc.NeoxcError, match="orbital 1"):
        F.read_mos(bad, 6)
    short = tmp_path / "short.dat"
    short.write_text("\n".join(txt[:5]) + "\n")
    with pytest.raises(neoxc.NeoxcError, match="ends at orbital 3"):
        F.read_mos(short, 6)
    with pytest.raises(neoxc.NeoxcError, match="cannot open"):
        F.read_mos(tmp_path / "missing.dat", 6)


@pytest.mark.parametrize("recl", [8, 32])
def test_ufm_layout(F, tmp_path, recl):
    """Record ia at byte (ia-1)*recl, the FP64 first, zero padding after."""
    v = np.random.default_rng(5).standard_normal(37)
    p = tmp_path / "GAM_ee.ufm"
    F.write_ufm(p, v, recl=recl)
    raw = np.fromfile(p, dtype="<f8")
    assert raw.size == 37 * recl // 8
    rec = raw.reshape(37, recl // 8)
    assert np.array_equal(rec[:, 0], v)
    assert not rec[:, 1:].any()
    assert np.array_equal(F.read_ufm(p, 37, recl=recl), v)


def test_ufm_recl_from_environment(F, tmp_path, monkeypatch):
    v = np.arange(6.0)
    p = tmp_path / "x.ufm"
    monkeypatch.setenv("NEOXC_UFM_RECL", "32")
    F.write_ufm(p, v)
    assert os.path.getsize(p) == 6 * 32
    assert np.array_equal(F.read_ufm(p, 6), v)
    monkeypatch.delenv("NEOXC_UFM_RECL")
    F.write_ufm(p, v)
    assert os.path.getsize(p) == 6 * 8


def test_ufm_short_file_is_an_error(F, tmp_path):
    import neoxc
    p = tmp_path / "s.ufm"
    F.write_ufm(p, np.ones(4), recl=8)
    with pytest.raises(neoxc.NeoxcError, match="4 of 5 records"):
        F.read_ufm(p, 5, recl=8)


def test_enuc_file(F, tmp_path):
    p = tmp_path / "ENUCRP.dat"
    F.write_enuc(p, 1.1412245162345678)
    assert F.read_enuc(p) == 1.1412245162345678
    # list-directed forms the Fortran write may produce
    p.write_text("   1.14122451623457     \n")
    assert F.read_enuc(p) == 1.14122451623457
    p.write_text(" 0.5D+00\n")
    assert F.read_enuc(p) == 0.5


def test_gam_io_shims(F, golden_xchf, in_tmp):
    """read_GAM_ee/ep/ecore/pcore, read_{elec,nuc}_ovlap, read_{elec,nuc}_
    density and write_MOs with the reference's names, arguments and files."""
    import neoxc
    L = neoxc.lib()
    rng = np.random.default_rng(9)
    ne, np_ = 3, 2
    gee, gep = rng.standard_normal(ne ** 4), rng.standard_normal(ne * ne * np_ * np_)
    ecr, pcr = rng.standard_normal(ne * ne), rng.standard_normal(np_ * np_)
    for name, v in (("GAM_ee.ufm", gee), ("GAM_ep.ufm", gep), ("GAM_ecr.ufm", ecr),
                    ("GAM_pcr.ufm", pcr)):
        F.write_ufm(name, v)

    def call(fn, *ints, n):
        out = np.zeros(n)
        getattr(L, fn)(*[_i64(i) for i in ints], out.ctypes.data_as(C.c_void_p))
        return out

    assert np.array_equal(call("read_gam_ee_", ne, ne ** 4, n=ne ** 4), gee)
    assert np.array_equal(call("read_gam_ep_", ne, np_, gep.size, n=gep.size), gep)
    assert np.array_equal(call("read_gam_ecore_", ne, ne * ne, n=ne * ne), ecr)
    assert np.array_equal(call("read_gam_pcore_", np_, np_ * np_, n=np_ * np_), pcr)
    # overlaps: GS(i,j) = record pack_2D(n,j,i) = j + n(i-1)
    S = rng.standard_normal((ne, ne))
    F.write_ufm("eovlap.ufm", S.ravel(order="F"))
    GS = call("read_elec_ovlap_", ne, n=ne * ne).reshape(ne, ne, order="F")
    assert np.array_equal(GS, S.T)
    Sp = rng.standard_normal((np_, np_))
    F.write_ufm("novlap.ufm", Sp.ravel(order="F"))
    assert np.array_equal(call("read_nuc_ovlap_", np_, n=np_ * np_).reshape(np_, np_, order="F"),
                          Sp.T)
    # densities from guessCE.inp / guessCP.inp
    open("guessCE.inp", "w").write(golden_xchf["guessCE"])
    V = F.read_mos("guessCE.inp", 6)
    DE = call("read_elec_density_", 6, 4, n=36).reshape(6, 6, order="F")
    assert np.abs(DE - 2.0 * V[:, :2] @ V[:, :2].T).max() <= 1e-15
    Vp = rng.standard_normal((3, 3))
    F.write_mos("guessCP.inp", Vp)
    Vp = F.read_mos("guessCP.inp", 3)
    DP = call("read_nuc_density_", 3, 1, 2, n=9).reshape(3, 3, order="F")
    assert np.abs(DP - np.outer(Vp[:, 1], Vp[:, 1])).max() <= 1e-15
    # write_MOs: unit -> file name
    for unit, name in ((852, "FinalCE.dat"), (853, "FinalCP.dat"), (860, "FinalCAE.dat"),
                       (861, "FinalCBE.dat"), (870, "FinalCAalpE.dat"),
                       (871, "FinalCAbetE.dat"), (999, "fort.999")):
        L.write_mos_(_i64(unit), _i64(6), V.ctypes.data_as(C.c_void_p))
        assert open(name).read() == golden_xchf["guessCE"], name

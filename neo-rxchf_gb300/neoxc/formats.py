"""The reference's on-disk formats (xchf1_independent/GAM_IO.f) through the
library's native readers and writers (``neoxc_ufm_*``, ``neoxc_mo_*``,
``neoxc_enuc_*`` in ``include/neoxc.h``).

* ``*.ufm`` -- direct-access integral files, one FP64 per record at the
  packed index (GAM_IO.f:1-245).  ``recl`` is the record length in bytes: 8
  when RECL=8 counts bytes (gfortran, ifort -assume byterecl), 32 for ifort's
  default 4-byte units; 0 reads ``NEOXC_UFM_RECL`` (default 8).
* MO files -- ``guessC*.inp`` (read, FORMAT(I2,I3,5E15.8)) and
  ``FinalC*.dat`` (PUSQLF, FORMAT(I2,I3,1P,5E15.8)), GAM_IO.f:247-518.
* ``ENUCRP.dat`` -- the classical nuclear repulsion energy
  (class_nuc_rep.f:39-41).

None of these touch the GPU.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _check, lib

# GAM_IO.f:1-26 unit map
UFM_FILES = {801: "GAM_1.ufm", 802: "GAM_1s.ufm", 803: "GAM_2.ufm", 804: "GAM_2s.ufm",
             805: "GAM_3.ufm", 806: "GAM_4.ufm", 810: "GAM_ee.ufm", 811: "GAM_ep.ufm",
             812: "GAM_ecr.ufm", 813: "GAM_pcr.ufm", 814: "eovlap.ufm",
             815: "novlap.ufm"}
MO_FILES = {850: "guessCE.inp", 851: "guessCP.inp", 852: "FinalCE.dat",
            853: "FinalCP.dat", 860: "FinalCAE.dat", 861: "FinalCBE.dat",
            870: "FinalCAalpE.dat", 871: "FinalCAbetE.dat"}


def _path(p) -> bytes:
    return os.fsencode(os.fspath(p))


def read_ufm(path, n: int, recl: int = 0) -> np.ndarray:
    """Records 1..n of a direct-access integral file (packed order)."""
    out = np.empty(n, dtype=np.float64)
    _check(lib().neoxc_ufm_read(_path(path), n, recl, out.ctypes.data))
    return out


def write_ufm(path, values, recl: int = 0) -> None:
    """Write `values` (packed order) as records 1..n."""
    v = np.ascontiguousarray(np.asarray(values, dtype=np.float64).ravel())
    _check(lib().neoxc_ufm_write(_path(path), v.ctypes.data, v.size, recl))


def write_mos(path, V) -> None:
    """PUSQLF (GAM_IO.f:471-518): V[:, j] is MO j, nbf = V.shape[0]."""
    V = np.asarray(V, dtype=np.float64)
    nbf, nmo = V.shape
    f = np.asfortranarray(V)
    _check(lib().neoxc_mo_write(_path(path), nbf, nmo, f.ctypes.data))


def read_mos(path, nbf: int, nmo: int | None = None) -> np.ndarray:
    """The VEC group of read_elec_density (GAM_IO.f:275-303): returns
    V(nbf, nmo) with V[:, j] = MO j; label mismatches raise NeoxcError."""
    nmo = nbf if nmo is None else nmo
    V = np.zeros((nbf, nmo), dtype=np.float64, order="F")
    _check(lib().neoxc_mo_read(_path(path), nbf, nmo, V.ctypes.data))
    return V


def mo_density(Cmo, kstart: int, klast: int, prefac: float) -> np.ndarray:
    """D = prefac * sum_{k=kstart..klast} C[:, k-1] C[:, k-1]^T (1-based k,
    GAM_IO.f:306-339)."""
    Cf = np.asfortranarray(np.asarray(Cmo, dtype=np.float64))
    n = Cf.shape[0]
    D = np.zeros((n, n), dtype=np.float64, order="F")
    _check(lib().neoxc_mo_density(n, kstart, klast, float(prefac), Cf.ctypes.data,
                                  D.ctypes.data))
    return D


def read_elec_density(path, nebf: int, n_particle: int) -> np.ndarray:
    """GAM_IO.f:247-347: the density of the nelec/2 lowest MOs (prefac 2),
    or of MO 1 (prefac 1) for a single particle."""
    V = read_mos(path, nebf)
    if n_particle > 1:
        return mo_density(V, 1, n_particle // 2, 2.0)
    return mo_density(V, 1, 1, 1.0)


def read_nuc_density(path, npbf: int, nucst: int) -> np.ndarray:
    """GAM_IO.f:349-448: the density of MO NUCST (prefac 1)."""
    return mo_density(read_mos(path, npbf), nucst, nucst, 1.0)


def write_enuc(path, E_nuc: float) -> None:
    _check(lib().neoxc_enuc_write(_path(path), float(E_nuc)))


def read_enuc(path) -> float:
    v = C.c_double()
    _check(lib().neoxc_enuc_read(_path(path), C.addressof(v)))
    return v.value

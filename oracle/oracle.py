"""ctypes binding for the CPU oracle (test infrastructure only).

The oracle restates the NEO-RXCHF integral and contraction arithmetic on
the CPU (``prim.c``, ``builders.c``, ``scf.c``, ``spin.c``, ``rx.c``).  Only the tests, the smoke check and
the CPU-baseline leg of ``bench.py`` load it; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libneoxc_oracle.so")
SOURCES = ["prim.c", "builders.c", "scf.c", "spin.c", "rx.c"]
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle (gcc, no FMA contraction, OpenMP) into _build/."""
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(HERE, "neoxc_oracle.h")]
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in srcs):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off",
           "-fno-fast-math", "-fopenmp", *[os.path.join(HERE, s) for s in SOURCES],
           "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class Prim(C.Structure):
    _fields_ = [("l", C.c_int * 3), ("a", C.c_double), ("c", C.c_double * 3)]


def prim(l, m, n, a, x, y, z) -> Prim:
    p = Prim()
    p.l[0], p.l[1], p.l[2] = int(l), int(m), int(n)
    p.a = float(a)
    p.c[0], p.c[1], p.c[2] = float(x), float(y), float(z)
    return p


class System(C.Structure):
    _fields_ = [
        ("nebf", C.c_int64), ("npebf", C.c_int64), ("npbf", C.c_int64),
        ("nat", C.c_int64), ("ngtg", C.c_int64),
        ("ELCAM", C.c_void_p), ("ELCEX", C.c_void_p), ("ELCBFC", C.c_void_p),
        ("AMPEB2C", C.c_void_p), ("AGEBFCC", C.c_void_p),
        ("KPESTR", C.c_void_p), ("KPEEND", C.c_void_p),
        ("NUCAM", C.c_void_p), ("NUCEX", C.c_void_p), ("NUCBFC", C.c_void_p),
        ("AGNBFCC", C.c_void_p), ("zan", C.c_void_p), ("cat", C.c_void_p),
        ("bgem", C.c_void_p), ("ggem", C.c_void_p), ("pmass", C.c_double),
    ]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB)
            d, i64, vp = C.c_double, C.c_int64, C.c_void_p
            P = C.POINTER(Prim)
            sig = {
                "orc_xgammaf": (None, [vp, d, C.c_int]),
                "orc_iboys2": (d, [C.c_int, d]),
                "orc_underflow": (d, [d]),
                "orc_rtuv": (d, [C.c_int] * 4 + [d] * 5),
                "orc_auxR2": (d, [C.c_int] * 3 + [d] * 4),
                "orc_gdel_x": (d, [C.c_int, d, d, d]),
                "orc_gfovlap": (d, [P, P]),
                "orc_gfke": (d, [P, P, d]),
                "orc_gfvec": (d, [P, P, vp]),
                "orc_gfvee": (d, [P, P, P, P]),
                "orc_g2_xggs": (d, [P, P, P, P, d, d]),
                "orc_g2_xggvec": (d, [P, P, P, P, d, d, vp]),
                "orc_g2_xggvee": (d, [P, P, P, P, d, d]),
                "orc_pgike1": (d, [P, P, P, P, d, d, d, vp]),
                "orc_g3_xggs": (d, [P, P, vp]),
                "orc_g3_ke": (d, [P, P, vp, d]),
                "orc_g3_xgvxcg": (d, [P, P, vp, vp]),
                "orc_g3_xgveeg": (d, [P, P, vp]),
                "orc_g4_xgveeg": (d, [P, P, d, d]),
                "orc_g4_xgvepg": (d, [P, P, d, d]),
                "orc_xcalc_gam2": (None, [P, P, vp, vp, vp]),
                "orc_xcalc_gam3": (d, [P, P, vp]),
                "orc_xcalc_gam2_rxchfne": (None, [P, P, vp, vp, vp]),
                "orc_pack_4d": (i64, [i64] * 7),
                "orc_index_gam_2pk": (i64, [i64] * 8),
                "orc_index_gam_3pk": (i64, [i64] * 10),
                "orc_index_gam_4pk2": (i64, [i64] * 12),
                "orc_loop_size": (None, [i64] * 4 + [vp, vp]),
                "orc_make_kpe": (None, [i64, i64, vp, vp, vp]),
                "orc_elcnorm3": (None, [i64, i64, vp, vp, vp, vp, vp]),
                "orc_nucnorm": (None, [i64, vp, vp, vp, vp]),
                "orc_gam2_raw": (None, [vp, i64, i64, vp, vp]),
                "orc_gam2_symmetrize": (None, [i64, i64, vp, vp, vp, vp]),
                "orc_gam2_ic1": (None, [vp, vp, vp]),
                "orc_gam3_raw": (None, [vp, i64, i64, vp]),
                "orc_gam3_symmetrize": (None, [i64, i64, vp, vp]),
                "orc_gam3_ic1": (None, [vp, vp]),
                "orc_contract_omega3": (d, [vp] + [i64] * 8),
                "orc_rxchfne_gam2_raw": (None, [vp, i64, i64, vp, vp]),
                "orc_rxchfne_gam2_ic1": (None, [vp, vp, vp]),
                "orc_calc_gam_ee": (None, [vp, vp]),
                "orc_gam4_element": (d, [i64, i64, vp, vp] + [i64] * 10),
                "orc_gam4_icr": (None, [i64, i64, vp, vp, vp]),
                "orc_gam4_dscf": (None, [i64, i64, vp, vp, vp, vp, vp, vp, vp]),
                "orc_gam4_dscf_range": (None, [i64, i64, vp, vp, vp, vp, i64, i64, vp, vp, vp]),
                "orc_gam4_dscf_sample": (None, [i64, i64, vp, vp, vp, vp, i64, i64, vp, vp, vp]),
                "orc_eg4icr": (None, [i64, i64, vp, vp, vp, vp, vp, vp]),
                "orc_eg3ic1": (None, [i64, i64, vp, vp, vp, vp, vp, vp]),
                "orc_eg2ic1": (None, [i64, i64] + [vp] * 10),
                "orc_rxchfne_fae_omg2": (None, [i64, i64] + [vp] * 6),
                "orc_rxchfne_fp_omg2": (None, [i64, i64] + [vp] * 6),
                "orc_rxchfne_fbe_omg2": (None, [i64, i64] + [vp] * 6),
                "orc_xcfock_correction": (None, [i64, i64, d, d] + [vp] * 6),
                "orc_density": (None, [i64, i64, d, vp, vp]),
                "orc_gam2_dscf": (None, [vp] + [vp] * 8),
                "orc_gam3_dscf": (None, [vp] + [vp] * 5),
                "orc_overlaps": (None, [vp] * 3),
                "orc_gam_epcore": (None, [vp] * 3),
                "orc_gam_ep": (None, [vp] * 2),
                "orc_gam1": (None, [vp] * 3),
                "orc_rxchf_gam1": (None, [vp] * 3),
                "orc_nuc_rep": (C.c_double, [vp]),
                "orc_num_threads": (C.c_int, []),
                "orc_gam4_raw": (d, [i64, i64, vp, vp] + [i64] * 10),
                "orc_fae_omg1": (None, [i64, i64] + [vp] * 8),
                "orc_ufp_omg1": (None, [i64, i64] + [vp] * 8),
                "orc_fae_omg2": (None, [i64] * 4 + [vp] * 9),
                "orc_ufp_omg2": (None, [i64] * 4 + [vp] * 9),
                "orc_fae_omg3": (None, [i64] * 4 + [vp] * 6),
                "orc_ufp_omg3": (None, [i64] * 4 + [vp] * 6),
                "orc_fae_omg4": (None, [i64] * 4 + [vp] * 6),
                "orc_ufp_omg4": (None, [i64] * 4 + [vp] * 6),
                "orc_fae_omg4_direct": (None, [i64] * 4 + [vp] * 7),
                "orc_ufp_omg4_direct": (None, [i64] * 4 + [vp] * 7),
                "orc_omg4_icr": (None, [i64, i64, vp, vp, vp]),
                "orc_rxcuhfne_fe_omg2": (None, [i64, i64] + [vp] * 9),
                "orc_rxcuhfne_fp_omg2": (None, [i64, i64] + [vp] * 8),
                "orc_rxcuhfne_fbe_omg2": (None, [i64, i64] + [vp] * 8),
                "orc_rxchf_fae_omg2": (None, [i64, i64] + [vp] * 10),
                "orc_rxchf_fp_omg2": (None, [i64, i64] + [vp] * 10),
                "orc_rxchf_fbe_omg2": (None, [i64, i64] + [vp] * 10),
                "orc_rxchf_fae_omg3": (None, [i64, i64] + [vp] * 7),
                "orc_rxchf_fp_omg3": (None, [i64, i64] + [vp] * 7),
                "orc_rxchf_fbe_omg3": (None, [i64, i64] + [vp] * 7),
                "orc_rxchf_fae_omg4": (None, [i64, i64] + [vp] * 6),
                "orc_rxchf_fp_omg4": (None, [i64, i64] + [vp] * 6),
                "orc_rxchf_fbe_omg4": (None, [i64, i64] + [vp] * 6),
                "orc_rxcuhf_fe_omg2": (None, [i64, i64] + [vp] * 12),
                "orc_rxcuhf_fp_omg2": (None, [i64, i64] + [vp] * 11),
                "orc_rxcuhf_fbe_omg2": (None, [i64, i64] + [vp] * 11),
                "orc_rxcuhf_fe_omg3": (None, [i64, i64] + [vp] * 10),
                "orc_rxcuhf_fp_omg3": (None, [i64, i64] + [vp] * 9),
                "orc_rxcuhf_fbe_omg3": (None, [i64, i64] + [vp] * 9),
            }
            for name, (res, args) in sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def prims(rows):
    arr = (Prim * len(rows))()
    for k, r in enumerate(rows):
        arr[k] = r if isinstance(r, Prim) else prim(*r)
    return arr


class SystemHandle:
    """Keeps the numpy arrays alive behind an ``orc_system`` struct."""

    def __init__(self, basis):
        self.b = basis  # neoxc.basis.NeoSystem-like object
        s = System()
        s.nebf, s.npebf, s.npbf = basis.nebf, basis.npebf, basis.npbf
        s.nat, s.ngtg = basis.nat, basis.ngtg
        self._keep = {}
        for name in ("ELCAM", "ELCEX", "ELCBFC", "AMPEB2C", "AGEBFCC", "KPESTR",
                     "KPEEND", "NUCAM", "NUCEX", "NUCBFC", "AGNBFCC", "zan", "cat",
                     "bgem", "ggem"):
            a = np.ascontiguousarray(getattr(basis, name + "_f"))
            self._keep[name] = a
            setattr(s, name, a.ctypes.data)
        s.pmass = float(basis.pmass)
        self.s = s

    @property
    def ref(self):
        return C.byref(self.s)

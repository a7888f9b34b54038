"""neoxc -- host-side mirror of the NEO-RXCHF geminal-integral routines on
the GB300 engine (``libneoxc_gb300.so``).

Every function here calls the C-ABI declared in ``include/neoxc.h``; the
names, argument meanings and output semantics follow the reference Fortran
routines they replace (builders return fresh arrays, Fock contractions
accumulate into the caller's matrices, energies are returned).  There is no
CPU implementation behind this module: if the library is missing or no
GB300 is usable, calls raise :class:`NeoxcError`.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build
from .basis import NeoSystem  # noqa: F401  (re-export)

__all__ = [
    "NeoxcError", "lib", "device_ok", "calc_gam_ee", "gam2_ic1", "gam3_ic1",
    "rxchfne_gam2_ic1", "gam4_icr", "gam4_dscf", "gam4_fock_factored",
    "gam3_dscf", "gam2_dscf", "xchf_scf", "xchf_scf_job", "xchf_scf_batch", "XchfServer",
    "SCF_SLOTS",
    "eg4icr", "eg3ic1", "eg2ic1",
    "rxchfne_fae_omg2", "rxchfne_fp_omg2", "rxchfne_fbe_omg2",
    "rxchfne_omg2_fused", "xcfock_correction", "index_map",
    "index_gam_2pk", "index_gam_3pk", "index_gam_4pk2", "pack_4d",
    "fae_omg1", "ufp_omg1", "fae_omg2", "ufp_omg2", "fae_omg3", "ufp_omg3", "fae_omg4",
    "ufp_omg4", "omg4_icr", "dev_xcuhf_omg", "dev_omg4_icr",
    "rxcuhfne_omg2", "rxchf_omg", "rxcuhf_omg", "rxchf_omg1", "xcuhf_scf", "XCUHF_SLOTS",
    "onebody_integrals", "class_nuc_rep", "xchf1_fock", "FOCK", "rx_scf", "RX_SLOTS", "rxchf_gam1", "rxchfne_fock",
]

LIB_PATH = _build.LIB
_lock = threading.Lock()
_lib = None


class NeoxcError(RuntimeError):
    """Error status returned by the GB300 library (message from
    neoxc_last_error)."""


def _declare(L):
    i64, d, vp = C.c_int64, C.c_double, C.c_void_p
    I = C.c_int
    sig = {
        "neoxc_last_error": (C.c_char_p, []),
        "neoxc_version": (I, []),
        "neoxc_device_ok": (I, []),
        "neoxc_pack_4d": (i64, [i64] * 7),
        "neoxc_index_gam_2pk": (i64, [i64] * 8),
        "neoxc_index_gam_3pk": (i64, [i64] * 10),
        "neoxc_index_gam_4pk2": (i64, [i64] * 12),
        "neoxc_index_map": (I, [i64, i64, i64, i64, vp]),
        "neoxc_make_kpe": (I, [i64, i64, vp, vp, vp]),
        "neoxc_calc_gam_ee": (I, [i64, i64, i64, vp, vp, vp, vp, vp, vp]),
        "neoxc_gam2_ic1": (I, [i64] * 8 + [d] + [vp] * 17),
        "neoxc_gam3_ic1": (I, [i64] * 8 + [d] + [vp] * 16),
        "neoxc_gam3_ic1_opts": (I, [i64] * 9 + [d] + [vp] * 17),
        "neoxc_gam3_ic1_batch": (I, [vp, i64, i64, vp, vp]),
        "neoxc_gam3_batch_tuning": (i64, [vp, i64]),
        "neoxc_set_mixed_threshold": (I, [d]),
        "neoxc_get_mixed_threshold": (d, []),
        "neoxc_rxchfne_gam2_ic1": (I, [i64] * 8 + [d] + [vp] * 17),
        "neoxc_gam3_dscf": (I, [i64] * 8 + [d] + [vp] * 20),
        "neoxc_gam2_dscf": (I, [i64] * 8 + [d] + [vp] * 23),
        "neoxc_gam4_icr": (I, [i64] * 6 + [vp] * 3),
        "neoxc_fae_omg1": (I, [i64] * 3 + [vp] * 8),
        "neoxc_ufp_omg1": (I, [i64] * 3 + [vp] * 8),
        "neoxc_fae_omg2": (I, [i64] * 6 + [vp] * 10),
        "neoxc_ufp_omg2": (I, [i64] * 6 + [vp] * 10),
        "neoxc_fae_omg3": (I, [i64] * 6 + [vp] * 6),
        "neoxc_ufp_omg3": (I, [i64] * 6 + [vp] * 6),
        "neoxc_fae_omg4": (I, [i64] * 6 + [vp] * 6),
        "neoxc_ufp_omg4": (I, [i64] * 6 + [vp] * 6),
        "neoxc_omg4_icr": (I, [i64] * 6 + [vp] * 3),
        "neoxc_rxcuhfne_fe_omg2": (I, [i64] * 4 + [vp] * 10),
        "neoxc_rxcuhfne_fp_omg2": (I, [i64] * 6 + [vp] * 8),
        "neoxc_rxcuhfne_fbe_omg2": (I, [i64] * 6 + [vp] * 8),
        "neoxc_rxchf_fae_omg2": (I, [i64] * 4 + [vp] * 10),
        "neoxc_rxchf_fp_omg2": (I, [i64] * 4 + [vp] * 10),
        "neoxc_rxchf_fbe_omg2": (I, [i64] * 4 + [vp] * 10),
        "neoxc_rxchf_fae_omg3": (I, [i64] * 4 + [vp] * 7),
        "neoxc_rxchf_fp_omg3": (I, [i64] * 4 + [vp] * 7),
        "neoxc_rxchf_fbe_omg3": (I, [i64] * 4 + [vp] * 7),
        "neoxc_rxchf_fae_omg4": (I, [i64] * 4 + [vp] * 6),
        "neoxc_rxchf_fp_omg4": (I, [i64] * 4 + [vp] * 6),
        "neoxc_rxchf_fbe_omg4": (I, [i64] * 4 + [vp] * 6),
        "neoxc_rxcuhf_fe_omg2": (I, [i64] * 4 + [vp] * 13),
        "neoxc_rxcuhf_fp_omg2": (I, [i64] * 6 + [vp] * 11),
        "neoxc_rxcuhf_fbe_omg2": (I, [i64] * 6 + [vp] * 11),
        "neoxc_rxcuhf_fe_omg3": (I, [i64] * 4 + [vp] * 10),
        "neoxc_rxcuhf_fp_omg3": (I, [i64] * 4 + [vp] * 9),
        "neoxc_rxcuhf_fbe_omg3": (I, [i64] * 4 + [vp] * 9),
        "neoxc_rxchf_fp_omg1": (I, [i64] * 3 + [vp] * 8),
        "neoxc_rxchf_fbe_omg1": (I, [i64] * 3 + [vp] * 8),
        "neoxc_dev_xcuhf_omg": (I, [vp] + [i64] * 5 + [vp] * 12),
        "neoxc_dev_omg4_icr": (I, [vp, i64, i64, vp, vp, vp]),
        "neoxc_gam4_dscf": (I, [i64] * 6 + [vp] * 7),
        "neoxc_gam4_fock_factored": (I, [i64] * 4 + [vp] * 7),
        "neoxc_xchf_scf": (I, [i64] * 7 + [d] + [vp] * 15 + [i64, i64] + [vp] * 7),
        "neoxc_xchf_job_size": (i64, []),
        "neoxc_xcuhf_scf": (I, [i64] * 9 + [d] + [vp] * 15 + [i64, i64] + [vp] * 8),
        "neoxc_xchf_scf_job": (I, [vp, i64, i64]),
        "neoxc_ufm_read": (I, [C.c_char_p, i64, i64, vp]),
        "neoxc_ufm_write": (I, [C.c_char_p, vp, i64, i64]),
        "neoxc_mo_write": (I, [C.c_char_p, i64, i64, vp]),
        "neoxc_mo_read": (I, [C.c_char_p, i64, i64, vp]),
        "neoxc_mo_density": (I, [i64, i64, i64, d, vp, vp]),
        "neoxc_enuc_write": (I, [C.c_char_p, d]),
        "neoxc_enuc_read": (I, [C.c_char_p, vp]),
        "neoxc_xchf_scf_batch": (I, [vp, i64, i64, i64, i64]),
        "neoxc_xchf_server_start": (vp, [i64, i64, i64]),
        "neoxc_xchf_server_submit": (I, [vp, vp]),
        "neoxc_xchf_server_set_budget": (I, [vp, i64]),
        "neoxc_admit": (I, [i64, i64, i64, i64]),
        "neoxc_xchf_job_bytes": (i64, [vp, i64]),
        "neoxc_xchf_server_wait": (I, [vp, vp, d]),
        "neoxc_xchf_server_stop": (I, [vp]),
        "neoxc_dev_gam4_fock_factored": (I, [vp, i64, i64] + [vp] * 7),
        "neoxc_dev_gam4_fock_factored_tc": (I, [vp, i64, i64] + [vp] * 7),
        "neoxc_eg4icr": (I, [i64] * 4 + [vp] * 6),
        "neoxc_eg3ic1": (I, [i64] * 4 + [vp] * 6),
        "neoxc_eg2ic1": (I, [i64] * 4 + [vp] * 10),
        "neoxc_rxchfne_fae_omg2": (I, [i64] * 4 + [vp] * 6),
        "neoxc_rxchfne_fp_omg2": (I, [i64] * 6 + [vp] * 6),
        "neoxc_rxchfne_fbe_omg2": (I, [i64] * 6 + [vp] * 6),
        "neoxc_rxchfne_omg2_fused": (I, [i64] * 2 + [vp] * 8),
        "neoxc_xcfock_correction": (I, [i64, i64, d, d, d] + [vp] * 6),
        "neoxc_onebody_integrals": (I, [i64] * 5 + [d] + [vp] * 20),
        "neoxc_class_nuc_rep": (I, [i64, vp, vp, vp]),
        "neoxc_rxchf_gam1": (I, [i64] * 7 + [d] + [vp] * 15),
        "neoxc_xchf1_fock": (I, [i64] * 13 + [vp] * 13 + [i64] * 4 + [d] + [vp] * 32),
        "neoxc_rx_scf": (I, [i64] * 10 + [d] + [vp] * 15 + [i64] + [vp] * 9),
        "neoxc_rxchfne_fock": (I, [i64] * 7 + [vp] * 20),
        "neoxc_probe_fp64": (I, [vp]),
        "neoxc_dev_gam4_dscf": (I, [vp, i64, i64] + [vp] * 7),
        "neoxc_dev_gam4_dscf_noalloc": (I, [vp, i64, i64] + [vp] * 7),
        "neoxc_dev_eg3ic1": (I, [vp, i64, i64] + [vp] * 6),
        "neoxc_dev_eg2ic1": (I, [vp, i64, i64] + [vp] * 10),
        "neoxc_dev_rxchfne_omg2": (I, [vp, i64, i64] + [vp] * 8),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def lib(build_if_missing: bool = False):
    """Load libneoxc_gb300.so.  Raises NeoxcError when it is absent."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                if build_if_missing:
                    _build.build()
                else:
                    raise NeoxcError(
                        "libneoxc_gb300.so is not built (run "
                        "`python -c 'import __graft_entry__ as g; g.build()'`); "
                        "there is no CPU fallback")
            L = C.CDLL(LIB_PATH)
            _declare(L)
            _lib = L
    return _lib


ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_UNSUPPORTED, ERR_IO, ERR_TIMEOUT, ERR_NUMERIC = 1, 2, 3, 4, 5, 6, 7
ADMIT_START, ADMIT_WAIT, ADMIT_REFUSE = 0, 1, 2


def _check(rc: int):
    if rc != 0:
        msg = lib().neoxc_last_error()
        raise NeoxcError("neoxc error %d: %s" % (rc, msg.decode() if msg else ""))


def device_ok() -> bool:
    return bool(lib().neoxc_device_ok())


def probe_fp64_tflops() -> float:
    """Measured FP64 FMA throughput of the current GPU (TFLOP/s)."""
    v = np.zeros(1)
    _check(lib().neoxc_probe_fp64(_p(v)))
    return float(v[0])


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _fmat(a) -> np.ndarray:
    """Column-major flat copy of a matrix (Fortran DE(n,n) layout)."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# ---- index maps (pack_GAM.f) --------------------------------------------
def pack_4d(n1, n2, n3, i1, i2, i3, i4) -> int:
    return int(lib().neoxc_pack_4d(n1, n2, n3, i1, i2, i3, i4))


def index_gam_2pk(nebf, npbf, ip, jp, ie1, je1, ie2, je2) -> int:
    return int(lib().neoxc_index_gam_2pk(nebf, npbf, ip, jp, ie1, je1, ie2, je2))


def index_gam_3pk(nebf, npbf, ip, jp, ie1, je1, ie2, je2, ie3, je3) -> int:
    return int(lib().neoxc_index_gam_3pk(nebf, npbf, ip, jp, ie1, je1, ie2, je2, ie3, je3))


def index_gam_4pk2(nebf, npbf, ip, jp, ie1, je1, ie2, je2, ie3, je3, ie4, je4) -> int:
    return int(lib().neoxc_index_gam_4pk2(nebf, npbf, ip, jp, ie1, je1, ie2, je2,
                                          ie3, je3, ie4, je4))


def index_map(kind: int, nebf: int, npbf: int, count: int | None = None) -> np.ndarray:
    """Whole packed-index map evaluated on the GPU, in the reference's loop
    order (kind 0: GAM_ee, 2/3/4: index_GAM_2PK/3PK/4PK2)."""
    total = {0: nebf ** 4, 2: nebf ** 4 * npbf ** 2, 3: nebf ** 6 * npbf ** 2,
             4: nebf ** 8 * npbf ** 2}[kind]
    n = total if count is None else count
    out = np.empty(n, np.int64)
    _check(lib().neoxc_index_map(kind, nebf, npbf, n, _p(out)))
    return out


# ---- builders ---------------------------------------------------------------
def _sysargs(s: NeoSystem):
    keep = [s.cat_f, s.zan_f, s.bgem_f, s.ggem_f, s.KPESTR_f, s.KPEEND_f,
            s.AMPEB2C_f, s.AGEBFCC_f, s.AGNBFCC_f, s.ELCEX_f, s.NUCEX_f,
            s.ELCAM_f, s.NUCAM_f, s.ELCBFC_f, s.NUCBFC_f]
    return keep, [_p(a) for a in keep]


def calc_gam_ee(s: NeoSystem) -> np.ndarray:
    """gam_ee.f calc_GAM_ee: contracted ERIs, packed pack_4D(je2,ie2,je1,ie1)."""
    out = np.empty(s.ngee)
    keep = [s.AMPEB2C_f, s.AGEBFCC_f, s.ELCEX_f, s.ELCAM_f, s.ELCBFC_f]
    _check(lib().neoxc_calc_gam_ee(s.nebf, s.npebf, s.ngee, *[_p(a) for a in keep], _p(out)))
    return out


def gam2_ic1(s: NeoSystem, nchunks: int = 1):
    """gam2_IC1_OMP.f GAM2_IC1 -> (GM2ICR, GM2sICR)."""
    g, gs = np.empty(s.ng2), np.empty(s.ng2)
    keep, ptrs = _sysargs(s)
    _check(lib().neoxc_gam2_ic1(nchunks, s.nebf, s.npebf, s.npbf, s.ng2, s.ng2prm,
                                s.nat, s.ngtg, s.pmass, *ptrs, _p(g), _p(gs)))
    return g, gs


def rxchfne_gam2_ic1(s: NeoSystem, nchunks: int = 1):
    """rxchfne_gam2_IC1_OMP.f RXCHFne_GAM2_IC1 -> (GM2ICR, GM2exICR)."""
    g, gx = np.empty(s.ng2), np.empty(s.ng2)
    keep, ptrs = _sysargs(s)
    _check(lib().neoxc_rxchfne_gam2_ic1(nchunks, s.nebf, s.npebf, s.npbf, s.ng2,
                                        s.ng2prm, s.nat, s.ngtg, s.pmass, *ptrs,
                                        _p(g), _p(gx)))
    return g, gx


def gam3_ic1(s: NeoSystem, nchunks: int = 1, mixed: bool = False, screen: bool = False,
             timing: bool = False):
    """gam3_IC1_OMP.f GAM3_IC1 -> GM3ICR.  mixed: four-particle terms with
    FP32 tables (FP64 Boys, seeds, sums); screen: skip primitive pairs below
    the 1e-12 Schwarz-type estimate; timing: also return the device seconds
    of the build."""
    g = np.empty(s.ng3)
    keep, ptrs = _sysargs(s)
    sec = np.zeros(1)
    opts = (8 if mixed else 0) | (64 if screen else 0)
    _check(lib().neoxc_gam3_ic1_opts(opts, nchunks, s.nebf, s.npebf, s.npbf, s.ng3, s.ng3prm,
                                     s.nat, s.ngtg, s.pmass, *ptrs, _p(g), _p(sec)))
    return (g, float(sec[0])) if timing else g


def gam3_dscf(s: NeoSystem, DE, DP, focke=None, fockp=None, nchunks: int = 1):
    """gam3_DSCF_OMP.f GAM3_DSCF: returns (focke + dF_e, fockp + dF_p, E_gam3)."""
    de, dp = _fmat(DE), _fmat(DP)
    fe, fp = _fock_io(s.nebf, s.npbf, focke, fockp)
    E = np.zeros(1)
    keep, ptrs = _sysargs(s)
    _check(lib().neoxc_gam3_dscf(nchunks, s.nebf, s.npebf, s.npbf, s.ng3, s.ng3prm,
                                 s.nat, s.ngtg, s.pmass, *ptrs, _p(de), _p(dp),
                                 _p(fe), _p(fp), _p(E)))
    return (*_fock_out(fe, fp, s.nebf, s.npbf), float(E[0]))


def gam2_dscf(s: NeoSystem, DE, DP, focke=None, fockp=None, se2=None, sp2=None,
              nchunks: int = 1):
    """gam2_DSCF_OMP.f GAM2_DSCF -> (focke, fockp, se2, sp2, E_gam2, S_gam2);
    the four matrices accumulate into the given ones (zeros when None)."""
    ne, np_ = s.nebf, s.npbf
    de, dp = _fmat(DE), _fmat(DP)
    fe, fp = _fock_io(ne, np_, focke, fockp)
    se, sp = _fock_io(ne, np_, se2, sp2)
    E, S = np.zeros(1), np.zeros(1)
    keep, ptrs = _sysargs(s)
    _check(lib().neoxc_gam2_dscf(nchunks, ne, s.npebf, np_, s.ng2, s.ng2prm,
                                 s.nat, s.ngtg, s.pmass, *ptrs, _p(de), _p(dp),
                                 _p(fe), _p(fp), _p(se), _p(sp), _p(E), _p(S)))
    return (*_fock_out(fe, fp, ne, np_), *_fock_out(se, sp, ne, np_),
            float(E[0]), float(S[0]))


# ---- one-body tables and the whole Fock build (xchf1_fock.f) --------------
ONEBODY = ("Se", "Sp", "GAM_ecore", "GAM_pcore", "GAM_ep", "GAM_1", "GAM_1s")


def onebody_integrals(s: NeoSystem, which=ONEBODY) -> dict:
    """elec_ovlap / nuc_ovlap (pure_ovlap.f), calc_GAM_epcore, calc_GAM_ep,
    GAM1_OMP_MD: each table in its file's record order (C-order [i][j] for
    the 2-index ones, [ip][jp][ie][je] for GAM_ep / GAM_1 / GAM_1s)."""
    ne, np_ = s.nebf, s.npbf
    size = {"Se": ne * ne, "Sp": np_ * np_, "GAM_ecore": ne * ne, "GAM_pcore": np_ * np_,
            "GAM_ep": s.ng1, "GAM_1": s.ng1, "GAM_1s": s.ng1}
    out = {k: np.empty(size[k]) for k in which}
    keep = [s.cat_f, s.zan_f, s.bgem_f, s.ggem_f, s.AMPEB2C_f, s.AGEBFCC_f, s.AGNBFCC_f,
            s.ELCEX_f, s.NUCEX_f, s.ELCAM_f, s.NUCAM_f, s.ELCBFC_f, s.NUCBFC_f]
    outs = [_p(out[k]) if k in out else None for k in ONEBODY]
    _check(lib().neoxc_onebody_integrals(ne, s.npebf, np_, s.nat, s.ngtg, s.pmass,
                                         *[_p(a) for a in keep], *outs))
    return out


def rxchf_gam1(s: NeoSystem):
    """rxchf_gam_1_OMP.f RXCHF_GAM1_OMP_MD -> (GAM_1, GAM_1s)."""
    g, gs = np.empty(s.ng1), np.empty(s.ng1)
    keep = [s.cat_f, s.zan_f, s.bgem_f, s.ggem_f, s.AMPEB2C_f, s.AGEBFCC_f, s.AGNBFCC_f,
            s.ELCEX_f, s.NUCEX_f, s.ELCAM_f, s.NUCAM_f, s.ELCBFC_f, s.NUCBFC_f]
    _check(lib().neoxc_rxchf_gam1(s.nebf, s.npebf, s.npbf, s.ng1,
                                  s.npebf ** 2 * s.npbf ** 2, s.nat, s.ngtg, s.pmass,
                                  *[_p(a) for a in keep], _p(g), _p(gs)))
    return g, gs


def class_nuc_rep(s: NeoSystem) -> float:
    """class_nuc_rep.f: classical nuclear repulsion."""
    E = np.zeros(1)
    _check(lib().neoxc_class_nuc_rep(s.nat, _p(s.zan_f), _p(s.cat_f), _p(E)))
    return float(E[0])


FOCK = {"neohf": 1, "gam4": 2, "g4dscf": 4, "g4ic": 8, "g3dscf": 16, "g3ic1": 32,
        "g2dscf": 64, "g2ic1": 128, "gam4_factored": 256}
FOCK_ENERGIES = ("E_total", "E_nuc", "E_ecore", "E_pcore", "E_ep", "E_ee", "E_gam1",
                 "E_gam2", "E_gam3", "E_gam4", "S_total", "S_gam1", "S_gam2")


def xchf1_fock(s: NeoSystem, DE, DP, tables: dict, E_nuc: float, modes=("gam4", "g4dscf",
               "g3ic1", "g2ic1"), nchunks: int = 1) -> dict:
    """xchf1_fock.f xchf1_fock on the device.  ``tables`` holds the arrays by
    their reference names (GAM_ecore, GAM_pcore, GAM_ep, GAM_ee, GAM_1,
    GAM_1s, GM2ICR, GM2SICR, GM3IC1, GM4ICR, GAM_2s; missing ones are passed
    as NULL); ``modes`` names the LOGICAL switches that are true (FOCK)."""
    ne, np_ = s.nebf, s.npbf
    m = 0
    for k in modes:
        m |= FOCK[k]
    de, dp = _fmat(DE), _fmat(DP)

    def t(name):
        v = tables.get(name)
        return None if v is None else np.ascontiguousarray(v, dtype=np.float64)

    names = ("GAM_ecore", "GAM_pcore", "GAM_ep", "GAM_ee", "GAM_1", "GAM_1s", "GM4ICR",
             "GM3IC1", "GM2ICR", "GM2SICR", "GAM_2s")
    tab = [t(n) for n in names]
    fe, fp, xfe, xfp = (np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(ne * ne),
                        np.zeros(np_ * np_))
    en = {k: np.zeros(1) for k in FOCK_ENERGIES}
    en["E_nuc"][0] = E_nuc
    keep, ptrs = _sysargs(s)
    _check(lib().neoxc_xchf1_fock(
        m, nchunks, nchunks, nchunks, s.npebf, ne, np_, s.nelec, s.ngee, s.ng1, s.ng2,
        s.ng3, s.ng4, _p(de), _p(dp), *[None if a is None else _p(a) for a in tab],
        s.ng2prm, s.ngtg, s.ng3prm, s.nat, s.pmass, *ptrs, _p(fe), _p(fp), _p(xfe),
        _p(xfp), *[_p(en[k]) for k in FOCK_ENERGIES]))
    out = {k: float(v[0]) for k, v in en.items()}
    out["focke"], out["fockp"] = _fock_out(fe, fp, ne, np_)
    out["Xfocke"], out["Xfockp"] = _fock_out(xfe, xfp, ne, np_)
    return out


RX_KINDS = {"rxchf_ne": 0, "rxcuhf_ne": 1, "rxcuhf_ae": 2}
RX_SLOTS = ("E_total", "E_nuc", "E_ecore", "E_ee", "E_OMG1", "E_OMG2", "S_total", "E_P_OMG1",
            "E_P_OMG2", "S_P_OMG1", "E_BE_OMG1", "S_BE_OMG1", "dDA", "dDBE", "dDP", "micro")


def rx_scf(s: NeoSystem, kind: str, nae: int = 0, nalp: int = 0, nbet: int = 0,
           nucst: int = 1, maxit: int = 100, ocbse: bool = True) -> dict:
    """One-special-electron RXCHF SCF on the device (rxchfne_scf.f
    xcrxchfne, rxcuhfne_scf.f xcrxcuhfne): kind "rxchf_ne" (nae closed-shell
    regular electrons), "rxcuhf_ne" or "rxcuhf_ae" (nalp alpha, nbet beta;
    EXCHLEV 0 / 1); ocbse=False selects the reference's LOCBSE = .false.
    branch.  Returns the initial and final energy slots (RX_SLOTS),
    the densities, the history and the iteration count."""
    ne, np_ = s.nebf, s.npbf
    DA, DB, DBE, DP = np.zeros(ne * ne), np.zeros(ne * ne), np.zeros(ne * ne), np.zeros(np_ * np_)
    Ei, Ef = np.zeros(16), np.zeros(16)
    hist = np.zeros(3 * maxit)
    nit, conv = C.c_int64(0), C.c_int64(0)
    keep, ptrs = _sysargs(s)
    _check(lib().neoxc_rx_scf(RX_KINDS[kind] | (0 if ocbse else 16), nae, nalp, nbet, nucst,
                              ne, s.npebf, np_, s.nat,
                              s.ngtg, s.pmass, *ptrs, maxit, _p(DA), _p(DB), _p(DBE), _p(DP),
                              _p(Ei), _p(Ef), _p(hist), C.byref(nit), C.byref(conv)))
    n = nit.value
    return {"initial": dict(zip(RX_SLOTS, Ei)), "final": dict(zip(RX_SLOTS, Ef)),
            "DA": DA.reshape(ne, ne, order="F"), "DAbet": DB.reshape(ne, ne, order="F"),
            "DBE": DBE.reshape(ne, ne, order="F"), "DP": DP.reshape(np_, np_, order="F"),
            "history": hist[:3 * n].reshape(n, 3), "niter": n, "converged": bool(conv.value)}


def rxchfne_fock(ne, np_, DA, DBE, DP, tables: dict, NAE=0, NAalpE=0, NAbetE=0, DAbet=None,
                 addexch=False) -> dict:
    """RXCHFne_FOCK (DAbet None) or RXCUHFne_FOCK on the device; ``tables``
    holds GAM_ecore, GAM_ee, GAM_1, GAM_1s, GM2ICR (and GM2exICR)."""
    open_ = DAbet is not None
    t = {k: None if tables.get(k) is None else np.ascontiguousarray(tables[k], dtype=np.float64)
         for k in ("GAM_ecore", "GAM_ee", "GAM_1", "GAM_1s", "GM2ICR", "GM2exICR")}
    da, dbe, dp = _fmat(DA), _fmat(DBE), _fmat(DP)
    db = _fmat(DAbet) if open_ else None
    FP, FA, FB, FBE = np.zeros(np_ * np_), np.zeros(ne * ne), np.zeros(ne * ne), np.zeros(ne * ne)
    en = [np.zeros(1) for _ in range(6)]

    def pp(a):
        return None if a is None else _p(a)
    _check(lib().neoxc_rxchfne_fock(int(open_), int(addexch), NAE, NAalpE, NAbetE, ne, np_,
                                    _p(da), pp(db), _p(dbe), _p(dp), pp(t["GAM_ecore"]),
                                    pp(t["GAM_ee"]), pp(t["GAM_1"]), pp(t["GAM_1s"]),
                                    pp(t["GM2ICR"]), pp(t["GM2exICR"]), _p(FP), _p(FA),
                                    _p(FB), _p(FBE), *[_p(e) for e in en]))
    r = dict(zip(("E_ecore", "E_ee", "E_OMG1", "E_OMG2", "E_total", "S_total"),
                 [float(e[0]) for e in en]))
    r["FP"], r["FAE"] = FP.reshape(np_, np_, order="F"), FA.reshape(ne, ne, order="F")
    r["FBE"] = FBE.reshape(ne, ne, order="F")
    if open_:
        r["FAbetE"] = FB.reshape(ne, ne, order="F")
    return r


SCF_SLOTS = ("E_total", "E_nuc", "E_ecore", "E_pcore", "E_ep", "E_ee", "E_gam1", "E_gam2",
             "E_gam3", "E_gam4", "S_total", "S_gam1", "S_gam2", "H_expect", "dDE", "dDP")


def xchf_scf(s: NeoSystem, DE, DP=None, nucst=None, maxit: int = 100,
             gam4_element: bool = False, diis: bool = False, mixed=False,
             screen: bool = False, soscf: bool = False):
    """xcscf.f XCHF RHF SCF on the GPU (plain Roothaan, or DIIS).  DE: initial
    electronic density, or None for the core-Hamiltonian guess (guess_elec);
    DP: initial nuclear density, or None for the core-Hamiltonian guess
    (guess_prot).  mixed: False (all FP64), "gam3" (FP32 MD integrals for
    gam_3), "gam2" (FP32 for gam_2, its large items in FP64: see
    set_mixed_threshold), True (both).
    screen: skip gam_3 primitive (bra, ket) pairs whose Schwarz-type
    estimate is below 1e-12 (NEOXC_SCF_SCREEN).  soscf: the reference's
    second-order steps on the electronic orbitals (NEOXC_SCF_SOSCF; not with
    diis).  Returns a dict with the initial and
    final energetics (SCF_SLOTS names), the per-iteration history, the
    converged densities, the iteration count and the convergence flag."""
    ne, np_ = s.nebf, s.npbf
    opts = ((1 if DP is None else 0) | (2 if diis else 0) | (4 if gam4_element else 0)
            | _mixed_bits(mixed) | (32 if DE is None else 0)
            | (64 if screen else 0) | (128 if soscf else 0))
    de = np.zeros(ne * ne) if DE is None else _fmat(DE).copy()
    dp = np.zeros(np_ * np_) if DP is None else _fmat(DP).copy()
    Ei, Ef = np.zeros(16), np.zeros(16)
    hist = np.zeros(4 * maxit)
    nit, conv = np.zeros(1, np.int64), np.zeros(1, np.int64)
    keep, ptrs = _sysargs(s)
    _check(lib().neoxc_xchf_scf(s.nelec, s.nucst if nucst is None else nucst, ne, s.npebf,
                                np_, s.nat, s.ngtg, s.pmass, *ptrs, opts, maxit, _p(de),
                                _p(dp), _p(Ei), _p(Ef), _p(hist), _p(nit), _p(conv)))
    n = int(nit[0])
    return {"initial": dict(zip(SCF_SLOTS, Ei.tolist())),
            "final": dict(zip(SCF_SLOTS, Ef.tolist())),
            "history": hist[:4 * n].reshape(n, 4), "niter": n, "converged": bool(conv[0]),
            "DE": de.reshape(ne, ne, order="F"), "DP": dp.reshape(np_, np_, order="F")}


XCUHF_SLOTS = ("E_total", "E_nuc", "E_ecore", "E_pcore", "E_ep", "E_ee", "E_omg1",
               "E_omg2", "E_omg3", "E_omg4", "S_total", "S_omg1", "S_omg2", "dDAE", "dDBE",
               "dDP")


def xcuhf_scf(s: NeoSystem, nae: int, nbe: int, DAE=None, DBE=None, DP=None, nucst=None,
              maxit: int = 100, diis: bool = False, mixed=False):
    """xcuhf_scf.f XCUHF SCF on the GPU (UROOTHAN for the proton, alpha and
    beta from each UHF_FOCK build; optional DIIS).  DAE / DBE None: core
    Hamiltonian guess for both spins (guess_A_elec); DP None: guess_prot2.
    Energies are the log's components (XCUHF_SLOTS, 2..9 divided by
    S_total).  Returns initial / final energetics, history, densities."""
    ne, np_ = s.nebf, s.npbf
    guess_e = DAE is None or DBE is None
    opts = ((1 if DP is None else 0) | (32 if guess_e else 0) | (2 if diis else 0)
            | _mixed_bits(mixed))
    da = np.zeros(ne * ne) if guess_e else _fmat(DAE).copy()
    db = np.zeros(ne * ne) if guess_e else _fmat(DBE).copy()
    dp = np.zeros(np_ * np_) if DP is None else _fmat(DP).copy()
    Ei, Ef, hist = np.zeros(16), np.zeros(16), np.zeros(4 * maxit)
    nit, conv = np.zeros(1, np.int64), np.zeros(1, np.int64)
    keep, ptrs = _sysargs(s)
    _check(lib().neoxc_xcuhf_scf(s.nelec, nae, nbe, s.nucst if nucst is None else nucst, ne,
                                 s.npebf, np_, s.nat, s.ngtg, s.pmass, *ptrs, opts, maxit,
                                 _p(da), _p(db), _p(dp), _p(Ei), _p(Ef), _p(hist), _p(nit),
                                 _p(conv)))
    n = int(nit[0])
    return {"initial": dict(zip(XCUHF_SLOTS, Ei.tolist())),
            "final": dict(zip(XCUHF_SLOTS, Ef.tolist())),
            "history": hist[:4 * n].reshape(n, 4), "niter": n, "converged": bool(conv[0]),
            "DAE": da.reshape(ne, ne, order="F"), "DBE": db.reshape(ne, ne, order="F"),
            "DP": dp.reshape(np_, np_, order="F")}


class XchfJob(C.Structure):
    """ctypes mirror of neoxc_xchf_job (include/neoxc.h)."""
    _fields_ = ([(n, C.c_int64) for n in ("nelec", "nucst", "nebf", "npebf", "npbf", "nat",
                                          "ngtg1")]
                + [("pmass", C.c_double)]
                + [(n, C.c_void_p) for n in ("cat", "zan", "bcoef1", "gamma1", "KPESTR",
                                             "KPEEND", "AMPEB2C", "AGEBFCC", "AGNBFCC",
                                             "ELCEX", "NUCEX", "ELCAM", "NUCAM", "ELCBFC",
                                             "NUCBFC", "DE", "DP", "E_init", "E_final",
                                             "history", "CE", "CP", "EE", "EP")]
                + [("niter", C.c_int64), ("converged", C.c_int64),
                   ("status", C.c_int32), ("reserved", C.c_int32),
                   ("t_submit", C.c_double), ("t_start", C.c_double),
                   ("t_end", C.c_double)])


def gam3_ic1_batch(systems, mixed: bool = False, screen: bool = False):
    """GAM3_IC1 for many systems through neoxc_gam3_ic1_batch (one
    persistent launch per angular class over a device work queue, grid
    chosen by the built-in autotuner).  Returns (list of GM3ICR arrays,
    device seconds of the build)."""
    n = len(systems)
    jobs = (XchfJob * n)()
    bufs = [_fill_job(jobs[k], s, np.eye(s.nebf), None, 1) for k, s in enumerate(systems)]
    outs = [np.empty(s.ng3) for s in systems]
    ptrs = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
    sec = np.zeros(1)
    opts = (8 if mixed else 0) | (64 if screen else 0)
    _check(lib().neoxc_gam3_ic1_batch(C.cast(jobs, C.c_void_p), n, opts, ptrs, _p(sec)))
    del bufs
    return outs, float(sec[0])


def set_mixed_threshold(tau: float) -> None:
    """neoxc_set_mixed_threshold: the contribution magnitude above which a
    mixed gam_2 primitive item is re-evaluated in FP64 (0: all, inf: none)."""
    _check(lib().neoxc_set_mixed_threshold(float(tau)))


def get_mixed_threshold() -> float:
    """neoxc_get_mixed_threshold."""
    return float(lib().neoxc_get_mixed_threshold())


def gam3_batch_tuning() -> list:
    """The autotuner's choices so far (neoxc_gam3_batch_tuning)."""
    import json
    n = lib().neoxc_gam3_batch_tuning(None, 0)
    buf = C.create_string_buffer(int(n) + 1)
    lib().neoxc_gam3_batch_tuning(buf, n + 1)
    return json.loads(buf.value.decode())


def xchf_scf_batch(systems, DEs, DPs=None, nworkers: int = 8, maxit: int = 100,
                   diis: bool = False, mixed=False, gam4_element: bool = False):
    """Independent XCHF solves through neoxc_xchf_scf_batch (worker threads
    with their own CUDA streams, memory-budget admission).  DPs: None for
    the core-Hamiltonian proton guess of every job.  Returns one result dict
    per system, as xchf_scf."""
    if C.sizeof(XchfJob) != lib().neoxc_xchf_job_size():
        raise NeoxcError("neoxc_xchf_job layout mismatch")
    opts = _scf_options(DPs is None, diis, mixed, gam4_element)
    n = len(systems)
    jobs = (XchfJob * n)()
    bufs = [_fill_job(jobs[k], s, DEs[k], None if DPs is None else DPs[k], maxit)
            for k, s in enumerate(systems)]
    _check(lib().neoxc_xchf_scf_batch(C.cast(jobs, C.c_void_p), n, nworkers, opts, maxit))
    return [_job_result(jobs[k], b) for k, b in enumerate(bufs)]


def _mixed_bits(mixed):
    """NEOXC_SCF_MIXED (8: gam_3) and NEOXC_SCF_MIXED_GAM2 (16: gam_2) for
    mixed = False, "gam3", "gam2" or True (both)."""
    if mixed not in (False, None, True, "gam3", "gam2"):
        raise ValueError("mixed: False, 'gam3', 'gam2' or True")
    return (8 if mixed in (True, "gam3") else 0) | (16 if mixed in (True, "gam2") else 0)


def _scf_options(guess_prot, diis, mixed, gam4_element):
    return ((1 if guess_prot else 0) | (2 if diis else 0) | (4 if gam4_element else 0)
            | _mixed_bits(mixed))


def _fill_job(j, s, DE, DP, maxit):
    """Point one neoxc_xchf_job at numpy buffers; returns the buffers (they
    must outlive the job)."""
    ne, np_ = s.nebf, s.npbf
    arrs, _ = _sysargs(s)
    de = _fmat(DE).copy()
    dp = np.zeros(np_ * np_) if DP is None else _fmat(DP).copy()
    Ei, Ef, hist = np.zeros(16), np.zeros(16), np.zeros(4 * maxit)
    CE, CP, EE, EP = np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(ne), np.zeros(np_)
    j.nelec, j.nucst, j.nebf, j.npebf, j.npbf = s.nelec, s.nucst, ne, s.npebf, np_
    j.nat, j.ngtg1, j.pmass = s.nat, s.ngtg, s.pmass
    names = ("cat", "zan", "bcoef1", "gamma1", "KPESTR", "KPEEND", "AMPEB2C", "AGEBFCC",
             "AGNBFCC", "ELCEX", "NUCEX", "ELCAM", "NUCAM", "ELCBFC", "NUCBFC")
    for name, a in zip(names, arrs):
        setattr(j, name, a.ctypes.data)
    j.DE, j.DP, j.E_init, j.E_final = de.ctypes.data, dp.ctypes.data, Ei.ctypes.data, Ef.ctypes.data
    j.history = hist.ctypes.data
    j.CE, j.CP, j.EE, j.EP = CE.ctypes.data, CP.ctypes.data, EE.ctypes.data, EP.ctypes.data
    return {"arrs": arrs, "ne": ne, "np": np_, "de": de, "dp": dp, "Ei": Ei, "Ef": Ef,
            "hist": hist, "CE": CE, "CP": CP, "EE": EE, "EP": EP}


def _job_result(j, b):
    nit = int(j.niter)
    return {"initial": dict(zip(SCF_SLOTS, b["Ei"].tolist())),
            "final": dict(zip(SCF_SLOTS, b["Ef"].tolist())),
            "history": b["hist"][:4 * nit].reshape(nit, 4), "niter": nit,
            "converged": bool(j.converged),
            "DE": b["de"].reshape(b["ne"], b["ne"], order="F"),
            "DP": b["dp"].reshape(b["np"], b["np"], order="F"),
            "CE": b["CE"].reshape(b["ne"], b["ne"], order="F"),
            "CP": b["CP"].reshape(b["np"], b["np"], order="F"),
            "EE": b["EE"].copy(), "EP": b["EP"].copy(),
            "t_submit": j.t_submit, "t_start": j.t_start, "t_end": j.t_end}


def xchf_scf_job(s: NeoSystem, DE, DP=None, maxit: int = 100, diis: bool = False,
                 mixed=False, gam4_element: bool = False):
    """One XCHF solve through neoxc_xchf_scf_job: as xchf_scf, plus the
    final MO coefficients CE, CP (columns by ascending orbital energy) and
    the orbital energies EE, EP."""
    job = XchfJob()
    bufs = _fill_job(job, s, DE, DP, maxit)
    _check(lib().neoxc_xchf_scf_job(C.byref(job),
                                    _scf_options(DP is None, diis, mixed, gam4_element),
                                    maxit))
    return _job_result(job, bufs)


class XchfServer:
    """Continuous-batching XCHF solves (neoxc_xchf_server_*): submit()
    queues a request and returns immediately; worker streams take requests
    as they free up; wait() returns the result dict (with the request's
    t_submit / t_start / t_end)."""

    def __init__(self, nworkers: int = 8, maxit: int = 100, diis: bool = True, mixed=True,
                 guess_prot: bool = True, gam4_element: bool = False):
        self.maxit, self.guess_prot = maxit, guess_prot
        self._h = lib().neoxc_xchf_server_start(
            nworkers, _scf_options(guess_prot, diis, mixed, gam4_element), maxit)
        if not self._h:
            raise NeoxcError(lib().neoxc_last_error().decode())

    def set_budget(self, cap_bytes: int):
        """Cap the device bytes the server's running jobs may hold together
        (0 = no cap beyond the free-memory rule of neoxc_admit)."""
        _check(lib().neoxc_xchf_server_set_budget(self._h, int(cap_bytes)))

    def submit(self, s: NeoSystem, DE, DP=None):
        job = XchfJob()
        bufs = _fill_job(job, s, DE, None if self.guess_prot else DP, self.maxit)
        _check(lib().neoxc_xchf_server_submit(self._h, C.byref(job)))
        return (job, bufs)

    def wait(self, ticket, timeout: float = 600.0, raise_on_error: bool = True):
        """The result dict once the request is done.  raise_on_error=False
        returns the dict with its "status" (NEOXC_ERR_NOMEM: refused,
        NEOXC_ERR_NUMERIC: non-finite energy) instead of raising; a timeout
        (NEOXC_ERR_TIMEOUT) always raises, and the request stays queued or
        running."""
        job, bufs = ticket
        rc = lib().neoxc_xchf_server_wait(self._h, C.byref(job), timeout)
        if rc == ERR_TIMEOUT or (rc != 0 and raise_on_error):
            _check(rc)
        r = _job_result(job, bufs)
        r["status"] = int(job.status)
        return r

    def stop(self):
        if self._h:
            _check(lib().neoxc_xchf_server_stop(self._h))
            self._h = None


def gam4_icr(ne: int, np_: int, gam_2s, gam_ee, nchunks: int = 1) -> np.ndarray:
    """gam4_ICR_OMP.f GAM4_ICR -> GAM_4 (gam_4/16, packed index_GAM_4PK2)."""
    g2, ge = _f64(gam_2s), _f64(gam_ee)
    ng4 = ne ** 8 * np_ ** 2
    out = np.empty(ng4)
    _check(lib().neoxc_gam4_icr(nchunks, ne, np_, ne ** 4, ne ** 4 * np_ ** 2, ng4,
                                _p(g2), _p(ge), _p(out)))
    return out


# ---- contractions ---------------------------------------------------------------
def _fock_io(ne, np_, focke, fockp):
    fe = np.zeros(ne * ne) if focke is None else _fmat(focke).copy()
    fp = np.zeros(np_ * np_) if fockp is None else _fmat(fockp).copy()
    return fe, fp


def _fock_out(fe, fp, ne, np_):
    return fe.reshape(ne, ne, order="F"), fp.reshape(np_, np_, order="F")


def gam4_dscf(ne, np_, gam_ee, gam_2s, DE, DP, focke=None, fockp=None, nchunks=1):
    """gam4_DSCF_OMP.f GAM4_DSCF: returns (focke + dF_e, fockp + dF_p, E_gam4)."""
    ge, g2, de, dp = _f64(gam_ee), _f64(gam_2s), _fmat(DE), _fmat(DP)
    fe, fp = _fock_io(ne, np_, focke, fockp)
    E = np.zeros(1)
    _check(lib().neoxc_gam4_dscf(nchunks, ne, np_, ne ** 4, ne ** 4 * np_ ** 2,
                                 ne ** 8 * np_ ** 2, _p(ge), _p(g2), _p(de), _p(dp),
                                 _p(fe), _p(fp), _p(E)))
    return (*_fock_out(fe, fp, ne, np_), float(E[0]))


def gam4_fock_factored(ne, np_, gam_ee, gam_2s, DE, DP, focke=None, fockp=None):
    """Factorised GAM4_DSCF Fock build (pair-symmetric tables): returns
    (focke + dF_e, fockp + dF_p, E_gam4)."""
    ge, g2, de, dp = _f64(gam_ee), _f64(gam_2s), _fmat(DE), _fmat(DP)
    fe, fp = _fock_io(ne, np_, focke, fockp)
    E = np.zeros(1)
    _check(lib().neoxc_gam4_fock_factored(ne, np_, ne ** 4, ne ** 4 * np_ ** 2, _p(ge),
                                          _p(g2), _p(de), _p(dp), _p(fe), _p(fp), _p(E)))
    return (*_fock_out(fe, fp, ne, np_), float(E[0]))


def eg4icr(ne, np_, DE, DP, gm4, focke=None, fockp=None, nchunks=1):
    """gam4_ICR_OMP.f EG4ICR."""
    g, de, dp = _f64(gm4), _fmat(DE), _fmat(DP)
    fe, fp = _fock_io(ne, np_, focke, fockp)
    E = np.zeros(1)
    _check(lib().neoxc_eg4icr(nchunks, ne, np_, len(g), _p(de), _p(dp), _p(g),
                              _p(fe), _p(fp), _p(E)))
    return (*_fock_out(fe, fp, ne, np_), float(E[0]))


def eg3ic1(ne, np_, DE, DP, gm3, focke=None, fockp=None, nchunks=1):
    """gam3_IC1_OMP.f EG3IC1."""
    g, de, dp = _f64(gm3), _fmat(DE), _fmat(DP)
    fe, fp = _fock_io(ne, np_, focke, fockp)
    E = np.zeros(1)
    _check(lib().neoxc_eg3ic1(nchunks, ne, np_, len(g), _p(de), _p(dp), _p(g),
                              _p(fe), _p(fp), _p(E)))
    return (*_fock_out(fe, fp, ne, np_), float(E[0]))


def eg2ic1(ne, np_, DE, DP, gm2, gm2s, FE=None, FP=None, nchunks=1):
    """gam2_IC1_OMP.f EG2IC1 -> (FE, SE, FP, SP, E_gam2, S_gam2)."""
    g, gs, de, dp = _f64(gm2), _f64(gm2s), _fmat(DE), _fmat(DP)
    fe, fp = _fock_io(ne, np_, FE, FP)
    se, sp = np.zeros(ne * ne), np.zeros(np_ * np_)
    E, S = np.zeros(1), np.zeros(1)
    _check(lib().neoxc_eg2ic1(nchunks, ne, np_, len(g), _p(de), _p(dp), _p(g), _p(gs),
                              _p(fe), _p(se), _p(fp), _p(sp), _p(E), _p(S)))
    return (fe.reshape(ne, ne, order="F"), se.reshape(ne, ne, order="F"),
            fp.reshape(np_, np_, order="F"), sp.reshape(np_, np_, order="F"),
            float(E[0]), float(S[0]))


def _omg2(fn, extra, ne, np_, DAE, DBE, DP, gm2, F, n):
    g, da, db, dp = _f64(gm2), _fmat(DAE), _fmat(DBE), _fmat(DP)
    f = np.zeros(n * n) if F is None else _fmat(F)
    E = np.zeros(1)
    _check(fn(1, ne, np_, len(g), *extra, _p(da), _p(db), _p(dp), _p(g), _p(f), _p(E)))
    return f.reshape(n, n, order="F"), float(E[0])


def rxchfne_fae_omg2(ne, np_, DAE, DBE, DP, gm2, FAE=None):
    """rxchfne_omg2.f RXCHFne_FAE_OMG2 -> (FAE, E_AE_OMG2)."""
    return _omg2(lib().neoxc_rxchfne_fae_omg2, (), ne, np_, DAE, DBE, DP, gm2, FAE, ne)


def rxchfne_fp_omg2(ne, np_, DAE, DBE, DP, gm2, FP=None, NAE=1, NBE=1):
    """rxchfne_omg2.f RXCHFne_FP_OMG2 -> (FP, E_P_OMG2)."""
    return _omg2(lib().neoxc_rxchfne_fp_omg2, (NAE, NBE), ne, np_, DAE, DBE, DP, gm2, FP, np_)


def rxchfne_fbe_omg2(ne, np_, DAE, DBE, DP, gm2, FBE=None, NAE=1, NBE=1):
    """rxchfne_omg2.f RXCHFne_FBE_OMG2 -> (FBE, E_BE_OMG2)."""
    return _omg2(lib().neoxc_rxchfne_fbe_omg2, (NAE, NBE), ne, np_, DAE, DBE, DP, gm2, FBE, ne)


def rxchfne_omg2_fused(ne, np_, DAE, DBE, DP, gm2):
    """One pass producing (FAE, FP, FBE, E_OMG2)."""
    g, da, db, dp = _f64(gm2), _fmat(DAE), _fmat(DBE), _fmat(DP)
    fa, fb, fp, E = np.zeros(ne * ne), np.zeros(ne * ne), np.zeros(np_ * np_), np.zeros(1)
    _check(lib().neoxc_rxchfne_omg2_fused(ne, np_, _p(da), _p(db), _p(dp), _p(g),
                                          _p(fa), _p(fp), _p(fb), _p(E)))
    return (fa.reshape(ne, ne, order="F"), fp.reshape(np_, np_, order="F"),
            fb.reshape(ne, ne, order="F"), float(E[0]))


# ---- open-shell XCUHF contractions (xcuhf/xcuhf_omg{1..4}.f) ---------------------
def fae_omg1(ne, np_, DAE, DP, gam1, gam1s, FAE=None):
    """xcuhf_omg1.f FAE_OMG1 -> (FAE + dF, SAE1, E_AE_OMG1, S_AE_OMG1)."""
    g, gs, da, dp = _f64(gam1), _f64(gam1s), _fmat(DAE), _fmat(DP)
    f = np.zeros(ne * ne) if FAE is None else _fmat(FAE).copy()
    sm, E, S = np.zeros(ne * ne), np.zeros(1), np.zeros(1)
    _check(lib().neoxc_fae_omg1(ne, np_, len(g), _p(da), _p(dp), _p(g), _p(gs), _p(f),
                                _p(sm), _p(E), _p(S)))
    return f.reshape(ne, ne, order="F"), sm.reshape(ne, ne, order="F"), float(E[0]), float(S[0])


def ufp_omg1(ne, np_, DETOT, DP, gam1, gam1s, FP=None):
    """xcuhf_omg1.f UFP_OMG1 -> (FP + dF, SP1, E_P_OMG1, S_P_OMG1)."""
    g, gs, dt, dp = _f64(gam1), _f64(gam1s), _fmat(DETOT), _fmat(DP)
    f = np.zeros(np_ * np_) if FP is None else _fmat(FP).copy()
    sm, E, S = np.zeros(np_ * np_), np.zeros(1), np.zeros(1)
    _check(lib().neoxc_ufp_omg1(ne, np_, len(g), _p(dt), _p(dp), _p(g), _p(gs), _p(f),
                                _p(sm), _p(E), _p(S)))
    return (f.reshape(np_, np_, order="F"), sm.reshape(np_, np_, order="F"), float(E[0]),
            float(S[0]))


def fae_omg2(ne, np_, NAE, NBE, DAE, DBE, DP, gm2, gm2s, FAE=None, nchunks=1):
    """xcuhf_omg2.f FAE_OMG2 -> (FAE + dF, SAE2, E_AE_OMG2, S_AE_OMG2)."""
    g, gs, da, db, dp = _f64(gm2), _f64(gm2s), _fmat(DAE), _fmat(DBE), _fmat(DP)
    dt = da + db
    f = np.zeros(ne * ne) if FAE is None else _fmat(FAE).copy()
    sm, E, S = np.zeros(ne * ne), np.zeros(1), np.zeros(1)
    _check(lib().neoxc_fae_omg2(nchunks, NAE, NBE, ne, np_, len(g), _p(da), _p(db), _p(dt),
                                _p(dp), _p(g), _p(gs), _p(f), _p(sm), _p(E), _p(S)))
    return f.reshape(ne, ne, order="F"), sm.reshape(ne, ne, order="F"), float(E[0]), float(S[0])


def ufp_omg2(ne, np_, NAE, NBE, DAE, DBE, DP, gm2, gm2s, FP=None, nchunks=1):
    """xcuhf_omg2.f UFP_OMG2 -> (FP + dF, SP2, E_P_OMG2, S_P_OMG2)."""
    g, gs, da, db, dp = _f64(gm2), _f64(gm2s), _fmat(DAE), _fmat(DBE), _fmat(DP)
    dt = da + db
    f = np.zeros(np_ * np_) if FP is None else _fmat(FP).copy()
    sm, E, S = np.zeros(np_ * np_), np.zeros(1), np.zeros(1)
    _check(lib().neoxc_ufp_omg2(nchunks, ne, np_, len(g), NAE, NBE, _p(da), _p(db), _p(dt),
                                _p(dp), _p(g), _p(gs), _p(f), _p(sm), _p(E), _p(S)))
    return (f.reshape(np_, np_, order="F"), sm.reshape(np_, np_, order="F"), float(E[0]),
            float(S[0]))


def _spin34(fn, n_out, ne, np_, NAE, NBE, DAE, DBE, DP, gm, F, nchunks):
    g, da, db, dp = _f64(gm), _fmat(DAE), _fmat(DBE), _fmat(DP)
    f = np.zeros(n_out * n_out) if F is None else _fmat(F).copy()
    E = np.zeros(1)
    _check(fn(nchunks, ne, np_, len(g), NAE, NBE, _p(da), _p(db), _p(dp), _p(g), _p(f),
              _p(E)))
    return f.reshape(n_out, n_out, order="F"), float(E[0])


def fae_omg3(ne, np_, NAE, NBE, DAE, DBE, DP, gm3, FAE=None, nchunks=1):
    """xcuhf_omg3.f FAE_OMG3 -> (FAE + dF, E_AE_OMG3)."""
    return _spin34(lib().neoxc_fae_omg3, ne, ne, np_, NAE, NBE, DAE, DBE, DP, gm3, FAE, nchunks)


def ufp_omg3(ne, np_, NAE, NBE, DAE, DBE, DP, gm3, FP=None, nchunks=1):
    """xcuhf_omg3.f UFP_OMG3 -> (FP + dF, E_P_OMG3)."""
    return _spin34(lib().neoxc_ufp_omg3, np_, ne, np_, NAE, NBE, DAE, DBE, DP, gm3, FP, nchunks)


def fae_omg4(ne, np_, NAE, NBE, DAE, DBE, DP, gm4, FAE=None, nchunks=1):
    """xcuhf_omg4.f FAE_OMG4 (gm4 from omg4_icr) -> (FAE + dF, E_AE_OMG4)."""
    return _spin34(lib().neoxc_fae_omg4, ne, ne, np_, NAE, NBE, DAE, DBE, DP, gm4, FAE, nchunks)


def ufp_omg4(ne, np_, NAE, NBE, DAE, DBE, DP, gm4, FP=None, nchunks=1):
    """xcuhf_omg4.f UFP_OMG4 -> (FP + dF, E_P_OMG4)."""
    return _spin34(lib().neoxc_ufp_omg4, np_, ne, np_, NAE, NBE, DAE, DBE, DP, gm4, FP, nchunks)


def omg4_icr(ne: int, np_: int, gam_2s, gam_ee, nchunks: int = 1) -> np.ndarray:
    """xcuhf_omg4.f OMG4_ICR -> the raw 5-particle tensor (index_GAM_4PK2)."""
    g2, ge = _f64(gam_2s), _f64(gam_ee)
    ng4 = ne ** 8 * np_ ** 2
    out = np.empty(ng4)
    _check(lib().neoxc_omg4_icr(nchunks, ne, np_, ne ** 4, ne ** 4 * np_ ** 2, ng4,
                                _p(g2), _p(ge), _p(out)))
    return out


def dev_xcuhf_omg(stream, K, ne, np_, NAE, NBE, d_G, d_Gs, d_DAE, d_DBE, d_DP,
                  d_FAE=None, d_FBE=None, d_FP=None, d_SAE=None, d_SBE=None, d_SP=None,
                  d_E=None):
    """FAE_OMGk (alpha and beta) and UFP_OMGk of rank K from one pass, on
    ``stream`` (torch float64 CUDA tensors; None skips an output)."""
    _check(lib().neoxc_dev_xcuhf_omg(C.c_void_p(stream), K, ne, np_, NAE, NBE,
                                     _tptr(d_G), _tptr(d_Gs), _tptr(d_DAE), _tptr(d_DBE),
                                     _tptr(d_DP), _tptr(d_FAE), _tptr(d_FBE), _tptr(d_FP),
                                     _tptr(d_SAE), _tptr(d_SBE), _tptr(d_SP), _tptr(d_E)))


# ---- special-electron contractions (rxchf/, rxchfne/) -----------------------------
def _rx_call(fn, lead, ne, np_, dens, tensors, outs, nen):
    """Call one RXCHF / RXCUHF routine: lead = the integer arguments before the
    arrays, outs = list of (n, initial matrix or None); returns
    (*matrices, *energies)."""
    arrs = [_fmat(d) for d in dens] + [_f64(t) for t in tensors]
    mats = [np.zeros(n * n) if F is None else _fmat(F).copy() for n, F in outs]
    ens = [np.zeros(1) for _ in range(nen)]
    _check(fn(*lead, *[_p(a) for a in arrs], *[_p(m) for m in mats], *[_p(e) for e in ens]))
    res = [m.reshape(n, n, order="F") for (n, _), m in zip(outs, mats)]
    return (*res, *[float(e[0]) for e in ens])


def rxcuhfne_omg2(which, ne, np_, DAalpE, DAbetE, DAtotE, DBE, DP, gm2, gm2ex, F=None,
                  F2=None, nchunks=1):
    """rxcuhfne_omg2.f RXCUHFne_FE_OMG2 ('fe': FAalpE, FAbetE, E), _FP_OMG2
    ('fp': FP, E) or _FBE_OMG2 ('fbe': FBE, E); F, F2 are added to."""
    ng = len(np.ravel(gm2))
    L = lib()
    if which == "fe":
        return _rx_call(L.neoxc_rxcuhfne_fe_omg2, (nchunks, ne, np_, ng), ne, np_,
                        (DAalpE, DAbetE, DAtotE, DBE, DP), (gm2, gm2ex),
                        [(ne, F), (ne, F2)], 1)
    fn = L.neoxc_rxcuhfne_fp_omg2 if which == "fp" else L.neoxc_rxcuhfne_fbe_omg2
    n = np_ if which == "fp" else ne
    return _rx_call(fn, (nchunks, ne, np_, ng, 0, 0), ne, np_, (DAalpE, DAtotE, DBE, DP),
                    (gm2, gm2ex), [(n, F)], 1)


def rxchf_omg(which, k, ne, np_, DAE, DBE, DP, tensors, F=None, S=None, nchunks=1):
    """rxchf_omg{2,3,4}.f RXCHF_{FAE,FP,FBE}_OMGk (which = 'fae', 'fp', 'fbe');
    tensors = (GM2_1ICR, GM2_2ICR, GM2sICR) | (GM3_1ICR, GM3_2ICR) | (GM4ICR,).
    Returns (F, S, E, S_E) for k = 2, else (F, E)."""
    ng = len(np.ravel(tensors[0]))
    fn = getattr(lib(), "neoxc_rxchf_%s_omg%d" % (which, k))
    n = np_ if which == "fp" else ne
    outs = [(n, F), (n, S)] if k == 2 else [(n, F)]
    return _rx_call(fn, (nchunks, ne, np_, ng), ne, np_, (DAE, DBE, DP), tensors, outs,
                    2 if k == 2 else 1)


def rxcuhf_omg(which, k, ne, np_, DAalpE, DAbetE, DAtotE, DBE, DP, tensors, F=None,
               F2=None, F3=None, nchunks=1):
    """rxcuhf_omg{2,3}.f RXCUHF_{FE,FP,FBE}_OMGk.  k = 2: 'fe' -> (FAalpE,
    FAbetE, SAalpE, E, S), 'fp' / 'fbe' -> (F, S, E, S_E); k = 3: 'fe' ->
    (FAalpE, FAbetE, E), 'fp' / 'fbe' -> (F, E)."""
    ng = len(np.ravel(tensors[0]))
    L = lib()
    fn = getattr(L, "neoxc_rxcuhf_%s_omg%d" % (which, k))
    n = np_ if which == "fp" else ne
    if k == 2:
        if which == "fe":
            return _rx_call(fn, (nchunks, ne, np_, ng), ne, np_,
                            (DAalpE, DAbetE, DAtotE, DBE, DP), tensors,
                            [(ne, F), (ne, F2), (ne, F3)], 2)
        return _rx_call(fn, (nchunks, ne, np_, ng, 0, 0), ne, np_, (DAalpE, DAtotE, DBE, DP),
                        tensors, [(n, F), (n, F2)], 2)
    outs = [(ne, F), (ne, F2)] if which == "fe" else [(n, F)]
    return _rx_call(fn, (nchunks, ne, np_, ng), ne, np_, (DAalpE, DAbetE, DAtotE, DBE, DP),
                    tensors, outs, 1)


def rxchf_omg1(which, ne, np_, DBE, DP, gam1, gam1s, F=None):
    """rxchf_omg1.f RXCHF_FP_OMG1 ('fp') / RXCHF_FBE_OMG1 ('fbe') ->
    (F + dF, S, E, S_E)."""
    g, gs, db, dp = _f64(gam1), _f64(gam1s), _fmat(DBE), _fmat(DP)
    n = np_ if which == "fp" else ne
    f = np.zeros(n * n) if F is None else _fmat(F).copy()
    sm, E, S = np.zeros(n * n), np.zeros(1), np.zeros(1)
    fn = lib().neoxc_rxchf_fp_omg1 if which == "fp" else lib().neoxc_rxchf_fbe_omg1
    _check(fn(ne, np_, len(g), _p(db), _p(dp), _p(g), _p(gs), _p(f), _p(sm), _p(E), _p(S)))
    return f.reshape(n, n, order="F"), sm.reshape(n, n, order="F"), float(E[0]), float(S[0])


def dev_omg4_icr(stream, ne, np_, d_gee, d_g2s, d_g4):
    """OMG4_ICR into the device tensor d_g4 (ne**8 np**2 float64) on ``stream``."""
    _check(lib().neoxc_dev_omg4_icr(C.c_void_p(stream), ne, np_, _tptr(d_gee), _tptr(d_g2s),
                                    _tptr(d_g4)))


def xcfock_correction(ne, np_, E_total, S_total, H_expect, se1, sp1, se2, sp2,
                      focke, fockp):
    """xchf1_fock.f XCfock_correction -> corrected (focke, fockp)."""
    a, b, c, d = _fmat(se1), _fmat(sp1), _fmat(se2), _fmat(sp2)
    fe, fp = _fmat(focke), _fmat(fockp)
    _check(lib().neoxc_xcfock_correction(ne, np_, E_total, S_total, H_expect, _p(a),
                                         _p(b), _p(c), _p(d), _p(fe), _p(fp)))
    return fe.reshape(ne, ne, order="F"), fp.reshape(np_, np_, order="F")


# ---- device-resident variants (torch CUDA tensors) --------------------------------
def _tptr(t):
    return C.c_void_p(None if t is None else t.data_ptr())


def dev_gam4_dscf(stream, ne, np_, d_gee, d_g2s, d_DE, d_DP, d_focke, d_fockp, d_E):
    """Enqueue the fused gam_4 direct-SCF contraction on ``stream`` (a raw
    cudaStream_t value); all arrays are torch float64 CUDA tensors."""
    _check(lib().neoxc_dev_gam4_dscf(C.c_void_p(stream), ne, np_, _tptr(d_gee),
                                     _tptr(d_g2s), _tptr(d_DE), _tptr(d_DP),
                                     _tptr(d_focke), _tptr(d_fockp), _tptr(d_E)))


def dev_gam4_fock_factored(stream, ne, np_, d_gee, d_g2s, d_DE, d_DP, d_focke, d_fockp, d_E):
    """Enqueue the factorised gam_4 Fock build on ``stream`` (pair-symmetric
    tables, not checked); all arrays are torch float64 CUDA tensors."""
    _check(lib().neoxc_dev_gam4_fock_factored(C.c_void_p(stream), ne, np_, _tptr(d_gee),
                                              _tptr(d_g2s), _tptr(d_DE), _tptr(d_DP),
                                              _tptr(d_focke), _tptr(d_fockp), _tptr(d_E)))


def dev_gam4_fock_factored_tc(stream, ne, np_, d_gee, d_g2s, d_DE, d_DP, d_focke, d_fockp,
                              d_E):
    """The factorised gam_4 Fock build with its transforms and focke
    contraction on the tensor cores (3xTF32, FP32 accumulation, FP64
    results); waits for the stream before returning."""
    _check(lib().neoxc_dev_gam4_fock_factored_tc(C.c_void_p(stream), ne, np_, _tptr(d_gee),
                                                 _tptr(d_g2s), _tptr(d_DE), _tptr(d_DP),
                                                 _tptr(d_focke), _tptr(d_fockp), _tptr(d_E)))


def dev_eg3ic1(stream, ne, np_, d_DE, d_DP, d_g3, d_focke, d_fockp, d_E):
    _check(lib().neoxc_dev_eg3ic1(C.c_void_p(stream), ne, np_, _tptr(d_DE), _tptr(d_DP),
                                  _tptr(d_g3), _tptr(d_focke), _tptr(d_fockp), _tptr(d_E)))


def dev_eg2ic1(stream, ne, np_, d_DE, d_DP, d_g2, d_g2s, d_FE, d_SE, d_FP, d_SP, d_E, d_S):
    _check(lib().neoxc_dev_eg2ic1(C.c_void_p(stream), ne, np_, _tptr(d_DE), _tptr(d_DP),
                                  _tptr(d_g2), _tptr(d_g2s), _tptr(d_FE), _tptr(d_SE),
                                  _tptr(d_FP), _tptr(d_SP), _tptr(d_E), _tptr(d_S)))


def dev_rxchfne_omg2(stream, ne, np_, d_DAE, d_DBE, d_DP, d_g2, d_FAE, d_FP, d_FBE, d_E):
    _check(lib().neoxc_dev_rxchfne_omg2(C.c_void_p(stream), ne, np_, _tptr(d_DAE),
                                        _tptr(d_DBE), _tptr(d_DP), _tptr(d_g2), _tptr(d_FAE),
                                        _tptr(d_FP), _tptr(d_FBE), _tptr(d_E)))

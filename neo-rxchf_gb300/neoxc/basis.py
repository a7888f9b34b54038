"""Host-side system description for the NEO-XCHF / RXCHF-ne hot path.

A :class:`NeoSystem` carries exactly the flat arrays the reference driver
(``xcneo_HYBRID.f``) hands to its integral builders, in Fortran layout:

* ``ELCAM(npebf,3)``, ``ELCEX(npebf)``, ``ELCBFC(npebf,3)``,
  ``AMPEB2C(npebf)``, ``AGEBFCC(npebf)``, ``KPESTR/KPEEND(nebf)``
  (xcneo_HYBRID.f:30-53, :398-430, make_KPE :1269-1307);
* ``NUCAM(npbf,3)``, ``NUCEX``, ``NUCBFC``, ``AGNBFCC`` (:432-445);
* ``zan(nat)``, ``cat(3,nat)`` (bohr, :375-389), geminal ``bgem/ggem``.

Attributes with an ``_f`` suffix are the 1-D column-major buffers passed
through the C-ABI.  Parsing covers the namelist input format of the
reference (``&SYSINFO``, ``&GEMINAL``, ``&ATOMS``, ``&EBASIS``, ``&PBASIS``)
and synthetic systems are generated with seeded numpy generators.
"""
from __future__ import annotations

import dataclasses
import math
import re
from typing import Optional

import numpy as np

A2BOHR = 1.0 / 0.529177249  # xcneo_HYBRID.f:97


@dataclasses.dataclass
class NeoSystem:
    nebf: int
    npebf: int
    npbf: int
    nat: int
    ngtg: int
    pmass: float
    nelec: int
    nucst: int
    ELCAM: np.ndarray    # (npebf,3) int64
    ELCEX: np.ndarray    # (npebf,)
    ELCBFC: np.ndarray   # (npebf,3) bohr
    AMPEB2C: np.ndarray  # (npebf,) 1-based
    AGEBFCC: np.ndarray  # (npebf,)
    KPESTR: np.ndarray   # (nebf,) 1-based
    KPEEND: np.ndarray   # (nebf,)
    NUCAM: np.ndarray    # (npbf,3)
    NUCEX: np.ndarray
    NUCBFC: np.ndarray   # (npbf,3)
    AGNBFCC: np.ndarray
    zan: np.ndarray      # (nat,)
    cat: np.ndarray      # (3,nat) bohr
    bgem: np.ndarray     # (ngtg,)
    ggem: np.ndarray     # (ngtg,)
    name: str = "system"

    # ---- Fortran-layout flat views -------------------------------------
    def _f(self, a, dtype):
        return np.ascontiguousarray(np.asarray(a, dtype=dtype).ravel(order="F"))

    @property
    def ELCAM_f(self): return self._f(self.ELCAM, np.int64)
    @property
    def ELCEX_f(self): return self._f(self.ELCEX, np.float64)
    @property
    def ELCBFC_f(self): return self._f(self.ELCBFC, np.float64)
    @property
    def AMPEB2C_f(self): return self._f(self.AMPEB2C, np.int64)
    @property
    def AGEBFCC_f(self): return self._f(self.AGEBFCC, np.float64)
    @property
    def KPESTR_f(self): return self._f(self.KPESTR, np.int64)
    @property
    def KPEEND_f(self): return self._f(self.KPEEND, np.int64)
    @property
    def NUCAM_f(self): return self._f(self.NUCAM, np.int64)
    @property
    def NUCEX_f(self): return self._f(self.NUCEX, np.float64)
    @property
    def NUCBFC_f(self): return self._f(self.NUCBFC, np.float64)
    @property
    def AGNBFCC_f(self): return self._f(self.AGNBFCC, np.float64)
    @property
    def zan_f(self): return self._f(self.zan, np.float64)
    @property
    def cat_f(self): return self._f(self.cat, np.float64)
    @property
    def bgem_f(self): return self._f(self.bgem, np.float64)
    @property
    def ggem_f(self): return self._f(self.ggem, np.float64)

    # ---- sizes (xcneo_HYBRID.f:463-473) ---------------------------------
    @property
    def ng1(self): return self.nebf ** 2 * self.npbf ** 2
    @property
    def ngee(self): return self.nebf ** 4
    @property
    def ng2(self): return self.nebf ** 4 * self.npbf ** 2
    @property
    def ng3(self): return self.nebf ** 6 * self.npbf ** 2
    @property
    def ng4(self): return self.nebf ** 8 * self.npbf ** 2
    @property
    def ng2prm(self): return self.npebf ** 4 * self.npbf ** 2
    @property
    def ng3prm(self): return self.npebf ** 6 * self.npbf ** 2

    def prims_per_contracted(self) -> np.ndarray:
        return (self.KPEEND - self.KPESTR + 1).astype(np.int64)


def make_kpe(nebf: int, ampeb2c: np.ndarray):
    """xcneo_HYBRID.f:1269-1307 make_KPE (contracted -> primitive ranges)."""
    kpestr = np.zeros(nebf, np.int64)
    kpeend = np.zeros(nebf, np.int64)
    ichk, ist = 1, 1
    npebf = len(ampeb2c)
    for iep in range(1, npebf + 1):
        iec = int(ampeb2c[iep - 1])
        if iec != ichk:
            ichk += 1
            kpestr[iec - 2] = ist
            kpeend[iec - 2] = iep - 1
            ist = iep
        if iep == npebf:
            kpestr[iec - 1] = ist
            kpeend[iec - 1] = iep
    return kpestr, kpeend


def _hermite_e0(i: int, j: int, a: float, b: float, ax: float, bx: float) -> float:
    """t=0 Hermite coefficient E^{ij}_0 (common.f:37-110 hecod)."""
    p = a + b
    q = a * b / p
    qx = ax - bx
    E = {(0, 0, 0): math.exp(-q * qx * qx)}
    c1, c2, d2 = 1.0 / (2.0 * p), -q * qx / a, q * qx / b

    def g(ii, jj, t):
        return E.get((ii, jj, t), 0.0)

    for ii in range(1, i + 1):
        for t in range(0, ii + 1):
            E[(ii, 0, t)] = c1 * g(ii - 1, 0, t - 1) + c2 * g(ii - 1, 0, t) + (t + 1) * g(ii - 1, 0, t + 1)
    for jj in range(1, j + 1):
        for ii in range(0, i + 1):
            for t in range(0, ii + jj + 1):
                E[(ii, jj, t)] = c1 * g(ii, jj - 1, t - 1) + d2 * g(ii, jj - 1, t) + (t + 1) * g(ii, jj - 1, t + 1)
    return E[(i, j, 0)]


def _ovlap(la, a, ca, lb, b, cb) -> float:
    """ovlap.f:2-70 gfovlap: product of 1-D E_0 sqrt(pi/p)."""
    s = 1.0
    for d in range(3):
        s *= _hermite_e0(int(la[d]), int(lb[d]), a, b, ca[d], cb[d]) * math.sqrt(math.pi / (a + b))
    return s


def elcnorm3(ampeb2c, agebfcc, elcex, elcam, elcbfc):
    """pure_ovlap.f:245-362 ELCNORM3 (primitive then contracted normalisation)."""
    c = np.array(agebfcc, dtype=np.float64)
    n = len(c)
    for i in range(n):
        c[i] = c[i] / math.sqrt(_ovlap(elcam[i], elcex[i], elcbfc[i], elcam[i], elcex[i], elcbfc[i]))
    nebf = int(max(ampeb2c))
    kappa = np.zeros(nebf)
    for i in range(n):
        for j in range(n):
            if ampeb2c[i] == ampeb2c[j]:
                kappa[ampeb2c[i] - 1] += _ovlap(elcam[i], elcex[i], elcbfc[i], elcam[j], elcex[j], elcbfc[j]) * c[i] * c[j]
    for i in range(n):
        c[i] = c[i] * (1.0 / math.sqrt(kappa[ampeb2c[i] - 1]))
    return c


def nucnorm(agnbfcc, nucex, nucam):
    """xcneo_HYBRID.f:1309-1347 NUCNORM."""
    c = np.array(agnbfcc, dtype=np.float64)
    z = (0.0, 0.0, 0.0)
    for i in range(len(c)):
        c[i] = c[i] * (1.0 / math.sqrt(_ovlap(nucam[i], nucex[i], z, nucam[i], nucex[i], z)))
    return c


# ---- reference input parser (namelist subset) --------------------------
def _nml_block(text: str, name: str) -> Optional[str]:
    m = re.search(r"&" + name + r"\b(.*?)/", text, re.S | re.I)
    return m.group(1) if m else None


def _nml_values(block: str) -> dict:
    out = {}
    for m in re.finditer(r"([A-Za-z_][A-Za-z_0-9]*)\s*(\(\s*\d+\s*\))?\s*=\s*([^,/\n]+)", block):
        key = m.group(1).lower()
        idx = m.group(2)
        val = m.group(3).strip()
        v = val.replace("d", "e").replace("D", "e")
        if val.upper() in (".T.", "T", ".TRUE."):
            pv = True
        elif val.upper() in (".F.", "F", ".FALSE."):
            pv = False
        else:
            try:
                pv = int(v)
            except ValueError:
                pv = float(v)
        if idx:
            out.setdefault(key, {})[int(idx.strip("() "))] = pv
        else:
            out[key] = pv
    return out


def _card_lines(text: str, card: str, n: int):
    lines = text.splitlines()
    for k, ln in enumerate(lines):
        if ln.strip().upper() == "&" + card:
            rows = [l for l in lines[k + 1:] if l.strip()][:n]
            return [r.split() for r in rows]
    raise ValueError("card &%s not found" % card)


def parse_inp(text: str, name: str = "input") -> NeoSystem:
    """Parse a reference ``*.inp`` (xcneo_HYBRID.f:120-445) and normalise the
    bases exactly as the driver does before any integral call."""
    sysinfo = _nml_values(_nml_block(text, "SYSINFO"))
    gem = _nml_values(_nml_block(text, "GEMINAL"))
    nat, nebf, npebf, npbf = (int(sysinfo[k]) for k in ("nat", "nebf", "npebf", "npbf"))
    ngtg = int(sysinfo["ngtg"])
    pmass = float(sysinfo.get("pmass", 1836.0))
    nelec = int(sysinfo.get("nelec", 2))
    nucst = int(sysinfo.get("nucst", 1))
    bgem = np.array([float(gem["bgem"][k]) for k in range(1, ngtg + 1)])
    ggem = np.array([float(gem["ggem"][k]) for k in range(1, ngtg + 1)])
    at = _card_lines(text, "ATOMS", nat)
    eb = _card_lines(text, "EBASIS", npebf)
    pb = _card_lines(text, "PBASIS", npbf)
    return _system(name, nebf, npebf, npbf, nat, ngtg, pmass, nelec, nucst, bgem, ggem,
                   at, eb, pb)


def _fnum(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "E"))


def parse_positional_inp(text: str, name: str = "input"):
    """Parse the older positional ``basis_definition.inp`` decks of the
    reference's tests/ directories: NGTG, NGTG rows of (b_k, gamma_k), NAT,
    NAT atom rows (Z, x, y, z in Angstrom, label), NEBF, NPEBF, NPEBF
    primitive rows (index, contracted index, l, m, n, exponent, coefficient,
    x, y, z in Angstrom), NPBF, NPBF nuclear rows alike, then one value per
    row tagged ``=NAME`` (PMASS, nelec, NAE, NBE, NUCST, the logical switches,
    EXCHLEV, NAalpE, NAbetE ...).  The logs of those runs echo the same
    parameters (coordinates converted to bohr).  Returns the normalised
    system and the tagged values keyed by lower-case name (strings)."""
    rows = [ln.split() for ln in text.splitlines() if ln.strip()]
    k = 0

    def take():
        nonlocal k
        k += 1
        return rows[k - 1]

    ngtg = int(take()[0])
    gem = [take() for _ in range(ngtg)]
    bgem = np.array([_fnum(r[0]) for r in gem])
    ggem = np.array([_fnum(r[1]) for r in gem])
    nat = int(take()[0])
    at = [take() for _ in range(nat)]
    nebf = int(take()[0])
    npebf = int(take()[0])
    eb = [take() for _ in range(npebf)]
    npbf = int(take()[0])
    pb = [take() for _ in range(npbf)]
    tags = {}
    for r in rows[k:]:
        line = " ".join(r)
        m = re.match(r"(\S+)\s*=\s*([A-Za-z_][A-Za-z_0-9]*)", line)
        if m and m.group(2).lower() not in tags:
            tags[m.group(2).lower()] = m.group(1)
    pmass = _fnum(tags.get("pmass", "1836.0"))
    nelec = int(tags.get("nelec", "2"))
    nucst = int(tags.get("nucst", "1"))
    sysm = _system(name, nebf, npebf, npbf, nat, ngtg, pmass, nelec, nucst, bgem, ggem,
                   at, eb, pb)
    return sysm, tags


def _system(name, nebf, npebf, npbf, nat, ngtg, pmass, nelec, nucst, bgem, ggem, at, eb,
            pb) -> NeoSystem:
    """Arrays of the driver (xcneo_HYBRID.f:375-445) from the ATOMS, EBASIS
    and PBASIS rows, with ELCNORM3 / NUCNORM applied."""
    zan = np.array([_fnum(r[0]) for r in at])
    cat = np.array([[A2BOHR * _fnum(r[d]) for r in at] for d in (1, 2, 3)])
    ampeb2c = np.array([int(r[1]) for r in eb], np.int64)
    elcam = np.array([[int(r[2]), int(r[3]), int(r[4])] for r in eb], np.int64)
    elcex = np.array([_fnum(r[5]) for r in eb])
    agebfcc = np.array([_fnum(r[6]) for r in eb])
    elcbfc = np.array([[A2BOHR * _fnum(r[7 + d]) for d in range(3)] for r in eb])
    nucam = np.array([[int(r[2]), int(r[3]), int(r[4])] for r in pb], np.int64)
    nucex = np.array([_fnum(r[5]) for r in pb])
    agnbfcc = np.array([_fnum(r[6]) for r in pb])
    nucbfc = np.array([[A2BOHR * _fnum(r[7 + d]) for d in range(3)] for r in pb])
    kpestr, kpeend = make_kpe(nebf, ampeb2c)
    agebfcc = elcnorm3(ampeb2c, agebfcc, elcex, elcam, elcbfc)
    agnbfcc = nucnorm(agnbfcc, nucex, nucam)
    return NeoSystem(nebf, npebf, npbf, nat, ngtg, pmass, nelec, nucst, elcam,
                     elcex, elcbfc, ampeb2c, agebfcc, kpestr, kpeend, nucam,
                     nucex, nucbfc, agnbfcc, zan, cat, bgem, ggem, name)


def read_mo_file(text: str, nbf: int) -> np.ndarray:
    """GAM_IO.f:247-300 reader of ``guessC*.inp`` / ``FinalC*.dat`` (format
    (I2,I3,5E15.8)); returns VEC(nbf,nbf) with VEC[:,j] = MO j."""
    vec = np.zeros((nbf, nbf))
    lines = [l for l in text.splitlines() if l.strip()]
    k = 0
    for j in range(nbf):
        imax = 0
        while imax < nbf:
            imin, imax = imax + 1, min(imax + 5, nbf)
            ln = lines[k]
            k += 1
            body = ln[5:]
            vals = [float(body[15 * q:15 * (q + 1)].replace("D", "E")) for q in range(imax - imin + 1)]
            vec[imin - 1:imax, j] = vals
    return vec


def density(vec: np.ndarray, nocc: int, prefac: float) -> np.ndarray:
    """GAM_IO.f:310-330: D(i,j) = sum_k prefac C(i,k) C(j,k), k <= nocc."""
    n = vec.shape[0]
    D = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            d = 0.0
            for k in range(nocc):
                d = d + prefac * vec[i, k] * vec[j, k]
            D[i, j] = d
    return D


# ---- seeded synthetic systems -------------------------------------------
def synthetic(seed: int, nat: int = 3, nebf: int = 12, nprim: int = 3,
              npbf: int = 8, ngtg: int = 3, lmax_e: int = 1, lmax_p: int = 2,
              e_exp=(0.1, 20.0), p_exp=(4.0, 32.0), gam=(0.5, 20.0),
              b=(0.1, 1.0), nelec: int = 4, name: str = "synthetic") -> NeoSystem:
    """Seeded random NEO system with the shapes of the XCHF/RXCHF-ne configs:
    nuclei uniform in [-1.5,1.5]^3 bohr, the quantum proton on nucleus 0,
    contracted Cartesian electronic shells with log-uniform exponents and
    uniform [0.1,1] coefficients (then normalised), an even-tempered nuclear
    basis on the proton centre, NG geminal terms (gamma log-uniform, b
    uniform).  ``nprim`` may be an int or an (lo,hi) range."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cat = rng.uniform(-1.5, 1.5, size=(3, nat))
    zan = np.ones(nat)
    zan[1:] = rng.integers(1, 4, size=nat - 1).astype(float)
    # electronic contracted functions: cycle s, px, py, pz (and d if lmax_e>=2)
    ams = [(0, 0, 0)]
    if lmax_e >= 1:
        ams += [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
    if lmax_e >= 2:
        ams += [(2, 0, 0), (1, 1, 0), (0, 2, 0), (1, 0, 1), (0, 1, 1), (0, 0, 2)]
    elcam, elcex, agebfcc, ampeb2c, elcbfc = [], [], [], [], []
    for ic in range(nebf):
        am = ams[ic % len(ams)]
        centre = cat[:, int(rng.integers(0, nat))]
        k = nprim if isinstance(nprim, int) else int(rng.integers(nprim[0], nprim[1] + 1))
        ex = np.exp(rng.uniform(math.log(e_exp[0]), math.log(e_exp[1]), size=k))
        co = rng.uniform(0.1, 1.0, size=k)
        for q in range(k):
            elcam.append(am)
            elcex.append(ex[q])
            agebfcc.append(co[q])
            ampeb2c.append(ic + 1)
            elcbfc.append(centre)
    npebf = len(elcex)
    pams = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (1, 1, 0),
            (0, 2, 0), (1, 0, 1), (0, 1, 1), (0, 0, 2)]
    pams = [a for a in pams if sum(a) <= lmax_p]
    nucam = np.array([pams[i % len(pams)] for i in range(npbf)], np.int64)
    ratio = (p_exp[1] / p_exp[0]) ** (1.0 / max(npbf - 1, 1))
    nucex = np.array([p_exp[0] * ratio ** i for i in range(npbf)])
    nucbfc = np.tile(cat[:, 0], (npbf, 1))
    agnbfcc = np.ones(npbf)
    ggem = np.exp(rng.uniform(math.log(gam[0]), math.log(gam[1]), size=ngtg))
    bgem = rng.uniform(b[0], b[1], size=ngtg)
    ampeb2c = np.array(ampeb2c, np.int64)
    elcam = np.array(elcam, np.int64)
    elcex = np.array(elcex)
    elcbfc = np.array(elcbfc)
    kpestr, kpeend = make_kpe(nebf, ampeb2c)
    agebfcc = elcnorm3(ampeb2c, np.array(agebfcc), elcex, elcam, elcbfc)
    agnbfcc = nucnorm(agnbfcc, nucex, nucam)
    return NeoSystem(nebf, npebf, npbf, nat, ngtg, 1836.0, nelec, 1, elcam,
                     elcex, elcbfc, ampeb2c, agebfcc, kpestr, kpeend, nucam,
                     nucex, nucbfc, agnbfcc, zan, cat, bgem, ggem, name)


def random_density(n: int, nocc: int, seed: int, prefac: float = 2.0) -> np.ndarray:
    """Seeded symmetric density from random orthonormal occupied orbitals."""
    rng = np.random.Generator(np.random.PCG64(seed))
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    c = q[:, :nocc] * 0.5
    return prefac * c @ c.T


def proton_scan(s: NeoSystem, n: int, amplitude: float = 0.5, seed: int = 0):
    """n copies of s with the quantum-proton basis centres displaced by a
    common seeded offset, uniform in [-amplitude, amplitude]^3 bohr (a
    proton-position scan; the classical nuclei and the electronic basis stay
    where they are)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        d = rng.uniform(-amplitude, amplitude, 3)
        out.append(dataclasses.replace(s, NUCBFC=np.asarray(s.NUCBFC, float) + d[None, :],
                                       name=s.name + "+scan"))
    return out

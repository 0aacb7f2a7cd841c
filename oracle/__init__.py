"""CPU checkers for the COORDINATION hot path.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.  It exposes two libraries through ctypes:

* ``Oracle`` -- ``_build/libcoord_oracle.so``, the plain-C FP64 restatement in
  ``coord_oracle.c`` (always buildable: only gcc is needed).
* ``Reference`` -- ``_ref/libcoord_ref.so``, the reference's own tool sources
  (src/tools/Pbc.cpp, SwitchingFunction.cpp, NeighborList.cpp, LinkCells.cpp,
  ...) compiled in place by ``Makefile`` with ``ref_harness.cpp`` driving them.
  Present only where the reference tree was available at build time.

Parity is pinned in two steps: ``Oracle`` == ``Reference`` bit for bit on the
same inputs (tests/test_oracle_vs_reference.py), and ``Oracle`` reproduces the
reference's regtest golden files (tests/test_oracle_golden.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libcoord_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libcoord_ref.so")
# the reference source tree (read only); PLUMED_REFERENCE_TREE overrides the default
REFERENCE_TREE = os.environ.get("PLUMED_REFERENCE_TREE", "/root/reference")

MODE_SINGLE, MODE_TWO, MODE_PAIR = 0, 1, 2
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def build(reference: bool | None = None, quiet: bool = True) -> None:
    """Compile the oracle (and the reference harness when the tree exists)."""
    targets = ["oracle"]
    if reference is None:
        reference = os.path.isdir(os.path.join(REFERENCE_TREE, "src", "tools"))
    if reference:
        targets.append("ref")
    out = subprocess.run(["make", "-s", "-j8", "-C", HERE, "REF=" + REFERENCE_TREE] + targets,
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


class _Pbc(C.Structure):
    _fields_ = [("type", C.c_int), ("box", C.c_double * 9), ("invbox", C.c_double * 9),
                ("reduced", C.c_double * 9), ("invreduced", C.c_double * 9),
                ("nshift", C.c_int * 8), ("shift", C.c_double * (8 * 32 * 3))]


class _Expr(C.Structure):  # orc_expr (orc_expr.h)
    _fields_ = [("ncode", C.c_int), ("code", C.c_int * 256), ("nconst", C.c_int), ("cst", C.c_double * 64),
                ("var_x2", C.c_int)]


class _Switch(C.Structure):
    _fields_ = [("type", C.c_int), ("d0", C.c_double), ("dmax", C.c_double), ("dmax_2", C.c_double),
                ("invr0", C.c_double), ("invr0_2", C.c_double), ("stretch", C.c_double),
                ("shift", C.c_double), ("nn", C.c_int), ("mm", C.c_int), ("preRes", C.c_double),
                ("preDfunc", C.c_double), ("preSecDev", C.c_double), ("nnf", C.c_int), ("mmf", C.c_int),
                ("preDfuncF", C.c_double), ("preSecDevF", C.c_double), ("a", C.c_int), ("b", C.c_int),
                ("c", C.c_double), ("d", C.c_double), ("beta", C.c_double), ("lambda_", C.c_double),
                ("ref", C.c_double), ("expr", _Expr)]


class _Pairing(C.Structure):
    _fields_ = [("kind", C.c_int), ("sw", C.c_void_p), ("dh_k", C.c_double), ("dh_constant", C.c_double),
                ("dh_epsilon", C.c_double), ("charge", C.c_void_p), ("gh_dmax_sq", C.c_double),
                ("gh_d0", C.c_double), ("gh_c_dmax2", C.c_double), ("gh_A", C.c_double), ("gh_B", C.c_double),
                ("gh_C", C.c_double), ("gh_D", C.c_double), ("gh_ntypes", C.c_int), ("type", C.c_void_p),
                ("eta", C.c_void_p)]


CV_COORDINATION, CV_DHENERGY, CV_GHBFIX = 0, 1, 2


# --- biases on a one-dimensional CV (numpy restatements) -------------------
METAD_DP2CUTOFF = 6.25  # Tools.h:71 (dp2cutoff)


def metad_hills(s, centres, sigmas, heights, stretch=True):
    """Sum of non-multivariate METAD hills at CV values s[f] and its derivative,
    MetaD::evaluateGaussianAndDerivatives (src/bias/MetaD.cpp:2256-2273):
    dp = (s - c)/sigma, dp2 = dp^2/2; a hill with dp2 < 6.25 adds
    h (A exp(-dp2) + B) to V and -A h exp(-dp2) dp/sigma to dV/ds, where A, B
    are the stretch constants of Tools.h:71-74 (A = 1, B = 0 unstretched).
    centres, sigmas, heights: [n_frames][n_hills]."""
    s = np.asarray(s, dtype=float)
    c, sg, h = (np.asarray(x, dtype=float) for x in (centres, sigmas, heights))
    e_cut = np.exp(-METAD_DP2CUTOFF)
    a = 1.0 / (1.0 - e_cut) if stretch else 1.0
    b = -e_cut / (1.0 - e_cut) if stretch else 0.0
    dp = (s[:, None] - c) / sg
    dp2 = 0.5 * dp * dp
    on = dp2 < METAD_DP2CUTOFF
    e = np.where(on, h * np.exp(-dp2), 0.0)
    V = (a * e + np.where(on, h * b, 0.0)).sum(1)
    dV = (-a * e * dp / sg).sum(1)
    return V, dV


def restraint(s, at, kappa, slope=0.0):
    """RESTRAINT on one argument, Restraint::calculate (src/bias/Restraint.cpp:
    125-141): V = kappa/2 (s-at)^2 + slope (s-at), dV/ds = kappa (s-at) + slope."""
    cv = np.asarray(s, dtype=float) - at
    return 0.5 * kappa * cv * cv + slope * cv, kappa * cv + slope


def _spec_is_r0(spec: str) -> bool:
    return spec.startswith("R0SYNTAX")


class Oracle:
    """ctypes wrapper of libcoord_oracle.so."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build(reference=False)
        L = C.CDLL(path)
        self.L = L
        L.orc_pbc_set.argtypes = [C.POINTER(_Pbc), _dp]
        L.orc_pbc_distance.argtypes = [C.POINTER(_Pbc), _dp, _dp, _dp]
        L.orc_tools_pbc.argtypes = [C.c_double]
        L.orc_tools_pbc.restype = C.c_double
        L.orc_switch_set.argtypes = [C.POINTER(_Switch), C.c_char_p, C.c_char_p, C.c_int]
        L.orc_switch_set_rational.argtypes = [C.POINTER(_Switch), C.c_int, C.c_int, C.c_double, C.c_double]
        for f in (L.orc_switch_calculate, L.orc_switch_calculate_sqr):
            f.argtypes = [C.POINTER(_Switch), C.c_double, C.POINTER(C.c_double)]
            f.restype = C.c_double
        L.orc_nl_nallpairs.argtypes = [C.c_int, C.c_int64, C.c_int64]
        L.orc_nl_nallpairs.restype = C.c_int64
        L.orc_nl_all_pairs.argtypes = [C.c_int, C.c_int64, C.c_int64, _u32p, C.c_int64]
        L.orc_nl_all_pairs.restype = C.c_int64
        for f in (L.orc_nl_classic, L.orc_nl_classic_cells, L.orc_nl_linkcells):
            f.argtypes = [C.c_int, C.c_int64, C.c_int64, _dp, C.POINTER(_Pbc), C.c_int, C.c_double,
                          _u32p, C.c_int64]
            f.restype = C.c_int64
        L.orc_linkcells_ncells.argtypes = [C.POINTER(_Pbc), C.c_double, C.POINTER(C.c_int * 3)]
        L.orc_linkcells_required.argtypes = [C.POINTER(_Pbc), C.c_double, C.POINTER(C.c_int * 3), C.c_int,
                                             C.POINTER(C.c_int * 27)]
        L.orc_linkcells_required.restype = C.c_int
        L.orc_coordination.argtypes = [C.POINTER(_Switch), C.POINTER(_Pbc), C.c_int, C.c_int64, _i64p, _dp,
                                       _u32p, C.c_int64, C.POINTER(C.c_double), _dp, _dp, C.c_int]
        L.orc_max_threads.restype = C.c_int
        L.orc_dhenergy_constants.argtypes = [C.c_double] * 6 + [C.POINTER(C.c_double)] * 2
        L.orc_ghbfix_constants.argtypes = [C.POINTER(_Pairing), C.c_double, C.c_double, C.c_double]
        L.orc_pairing_eval.argtypes = [C.POINTER(_Pairing), C.c_double, C.POINTER(C.c_double), C.c_int64,
                                       C.c_int64]
        L.orc_pairing_eval.restype = C.c_double
        L.orc_cv.argtypes = [C.POINTER(_Pairing), C.POINTER(_Pbc), C.c_int, C.c_int64, _i64p, _dp, _u32p,
                             C.c_int64, C.POINTER(C.c_double), _dp, _dp, C.c_int]
        L.orc_contactmap.argtypes = [C.c_void_p, C.c_int, C.c_int64, _dp, _dp, C.c_int, C.POINTER(_Pbc), C.c_int, _dp,
                                     _dp, _dp, _dp]
        L.orc_peratom.argtypes = [C.POINTER(_Switch), C.POINTER(_Pbc), C.c_int, C.c_int64, _i64p, _dp, _u32p,
                                  C.c_int64, C.c_void_p, _dp, C.c_void_p, C.c_void_p]

    # -- pbc -----------------------------------------------------------------
    def pbc(self, box) -> _Pbc:
        p = _Pbc()
        self.L.orc_pbc_set(C.byref(p), np.ascontiguousarray(np.asarray(box, np.float64).reshape(9)))
        return p

    def pbc_distance(self, box, v1, v2) -> np.ndarray:
        p = self.pbc(box)
        v1 = np.ascontiguousarray(np.asarray(v1, np.float64).reshape(-1, 3))
        v2 = np.ascontiguousarray(np.asarray(v2, np.float64).reshape(-1, 3))
        out = np.empty_like(v1)
        d = np.empty(3)
        for i in range(len(v1)):
            self.L.orc_pbc_distance(C.byref(p), v1[i].copy(), v2[i].copy(), d)
            out[i] = d
        return out

    # -- switching functions -------------------------------------------------
    def switch(self, spec: str) -> _Switch:
        s = _Switch()
        if _spec_is_r0(spec):
            nn, mm, r0, d0 = spec.split()[1:]
            self.L.orc_switch_set_rational(C.byref(s), int(nn), int(mm), float(r0), float(d0))
            return s
        err = C.create_string_buffer(512)
        if self.L.orc_switch_set(C.byref(s), spec.encode(), err, 512):
            raise ValueError(err.value.decode())
        return s

    def switch_eval(self, spec: str, x, squared: bool = True):
        s = self.switch(spec)
        f = np.empty(len(x))
        df = np.empty(len(x))
        d = C.c_double()
        fn = self.L.orc_switch_calculate_sqr if squared else self.L.orc_switch_calculate
        for i, v in enumerate(np.asarray(x, np.float64)):
            f[i] = fn(C.byref(s), float(v), C.byref(d))
            df[i] = d.value
        return f, df

    # -- neighbour lists -----------------------------------------------------
    def nallpairs(self, mode, n0, n1=0) -> int:
        return self.L.orc_nl_nallpairs(mode, n0, n1)

    def all_pairs(self, mode, n0, n1=0) -> np.ndarray:
        n = self.nallpairs(mode, n0, n1)
        out = np.empty(2 * max(n, 1), np.uint32)
        self.L.orc_nl_all_pairs(mode, n0, n1, out, n)
        return out[:2 * n].reshape(-1, 2)

    def _nl(self, fn, mode, n0, n1, pos, box, do_pbc, cutoff, cap=None):
        pos = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(-1, 3))
        p = self.pbc(box)
        cap = cap or max(1024, 64 * len(pos))
        while True:
            out = np.empty(2 * cap, np.uint32)
            n = fn(mode, n0, n1, pos.reshape(-1), C.byref(p), int(do_pbc), float(cutoff), out, cap)
            if n == -2:
                raise ValueError("Cell lists cannot be built when passing a box with null volume")
            if n < 0:
                raise ValueError("this neighbour-list builder does not take PAIR mode")
            if n <= cap:
                return out[:2 * n].reshape(-1, 2)
            cap = int(n)

    def nl_classic(self, mode, n0, n1, pos, box, do_pbc, cutoff):
        return self._nl(self.L.orc_nl_classic, mode, n0, n1, pos, box, do_pbc, cutoff)

    def nl_classic_cells(self, mode, n0, n1, pos, box, do_pbc, cutoff):
        return self._nl(self.L.orc_nl_classic_cells, mode, n0, n1, pos, box, do_pbc, cutoff)

    def nl_linkcells(self, mode, n0, n1, pos, box, do_pbc, cutoff):
        return self._nl(self.L.orc_nl_linkcells, mode, n0, n1, pos, box, do_pbc, cutoff)

    def linkcells_ncells(self, box, cutoff):
        nc = (C.c_int * 3)()
        p = self.pbc(box)
        self.L.orc_linkcells_ncells(C.byref(p), float(cutoff), C.byref(nc))
        return list(nc)

    def linkcells_required(self, box, cutoff, cell, use_pbc=True):
        """Sorted indices of the cells searched from the cell with indices cell."""
        req = (C.c_int * 27)()
        p = self.pbc(box)
        n = self.L.orc_linkcells_required(C.byref(p), float(cutoff), C.byref((C.c_int * 3)(*cell)), int(use_pbc),
                                          C.byref(req))
        return sorted(req[:n])

    # -- the CV ----------------------------------------------------------------
    def coordination(self, spec, pos, box, pairs, abs_index=None, do_pbc=True, nthreads=1):
        """s, derivatives (nslots x 3) and virial (3 x 3) over the given pairs."""
        pos = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(-1, 3))
        n = len(pos)
        if abs_index is None:
            abs_index = np.arange(n, dtype=np.int64)
        abs_index = np.ascontiguousarray(abs_index, dtype=np.int64)
        pairs = np.ascontiguousarray(np.asarray(pairs, np.uint32).reshape(-1, 2))
        sw = self.switch(spec)
        p = self.pbc(box)
        s = C.c_double()
        deriv = np.zeros(3 * n)
        vir = np.zeros(9)
        self.L.orc_coordination(C.byref(sw), C.byref(p), int(do_pbc), n, abs_index, pos.reshape(-1),
                                pairs.reshape(-1) if len(pairs) else np.zeros(2, np.uint32), len(pairs),
                                C.byref(s), deriv, vir, int(nthreads))
        return s.value, deriv.reshape(n, 3), vir.reshape(3, 3)

    # -- sibling CVs (DHENERGY, GHBFIX) -----------------------------------------
    def dhenergy_constants(self, ionic, temp, epsilon, unit_energy=1.0, unit_length=1.0, unit_charge=1.0):
        """(k, constant) of DHEnergy::DHEnergy (DHEnergy.cpp:112-113)."""
        k, c = C.c_double(), C.c_double()
        self.L.orc_dhenergy_constants(ionic, temp, epsilon, unit_energy, unit_length, unit_charge, C.byref(k),
                                      C.byref(c))
        return k.value, c.value

    def pairing(self, kind, *, charges=None, dh=None, types=None, eta=None, ghbfix=None):
        """A pairing descriptor.  DHENERGY: charges per slot and dh = (k, constant,
        epsilon).  GHBFIX: types per slot, eta (n x n) and ghbfix = (d0, dmax, c).
        The arrays are kept alive on the returned object."""
        p = _Pairing()
        p.kind = kind
        keep = []
        if kind == CV_DHENERGY:
            q = np.ascontiguousarray(charges, np.float64)
            keep.append(q)
            p.charge = q.ctypes.data
            p.dh_k, p.dh_constant, p.dh_epsilon = dh
        elif kind == CV_GHBFIX:
            t = np.ascontiguousarray(types, np.int32)
            e = np.ascontiguousarray(eta, np.float64)
            keep += [t, e]
            p.type, p.eta = t.ctypes.data, e.ctypes.data
            p.gh_ntypes = int(round(np.sqrt(e.size)))
            self.L.orc_ghbfix_constants(C.byref(p), *[float(v) for v in ghbfix])
        p._keep = keep
        return p

    def pairing_eval(self, p, r2, i, j):
        df = C.c_double()
        f = self.L.orc_pairing_eval(C.byref(p), float(r2), C.byref(df), int(i), int(j))
        return f, df.value

    def cv(self, p, pos, box, pairs, abs_index=None, do_pbc=True, nthreads=1):
        """CoordinationBase::calculate with pairing p: s, derivatives, virial."""
        pos = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(-1, 3))
        n = len(pos)
        if abs_index is None:
            abs_index = np.arange(n, dtype=np.int64)
        abs_index = np.ascontiguousarray(abs_index, dtype=np.int64)
        pairs = np.ascontiguousarray(np.asarray(pairs, np.uint32).reshape(-1, 2))
        pb = self.pbc(box)
        s = C.c_double()
        deriv = np.zeros(3 * n)
        vir = np.zeros(9)
        self.L.orc_cv(C.byref(p), C.byref(pb), int(do_pbc), n, abs_index, pos.reshape(-1),
                      pairs.reshape(-1) if len(pairs) else np.zeros(2, np.uint32), len(pairs), C.byref(s), deriv,
                      vir, int(nthreads))
        return s.value, deriv.reshape(n, 3), vir.reshape(3, 3)

    def peratom(self, spec, pos, box, pairs, abs_index=None, do_pbc=True, g=None):
        """Per-atom coordination over the given pairs (CONTACT_MATRIX x ones):
        cn per slot; with g (dV/dcn per slot) also (grad (nslots x 3), virial 3x3)."""
        pos = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(-1, 3))
        n = len(pos)
        if abs_index is None:
            abs_index = np.arange(n, dtype=np.int64)
        abs_index = np.ascontiguousarray(abs_index, dtype=np.int64)
        pairs = np.ascontiguousarray(np.asarray(pairs, np.uint32).reshape(-1, 2))
        sw = self.switch(spec)
        pb = self.pbc(box)
        cn = np.zeros(n)
        grad = np.zeros(3 * n)
        vir = np.zeros(9)
        gg = None if g is None else np.ascontiguousarray(g, np.float64)
        self.L.orc_peratom(C.byref(sw), C.byref(pb), int(do_pbc), n, abs_index, pos.reshape(-1),
                           pairs.reshape(-1) if len(pairs) else np.zeros(2, np.uint32), len(pairs),
                           None if gg is None else gg.ctypes.data, cn, None if gg is None else grad.ctypes.data,
                           None if gg is None else vir.ctypes.data)
        if gg is None:
            return cn
        return cn, grad.reshape(n, 3), vir.reshape(3, 3)

    def contactmap(self, specs, pos, box, reference=None, weight=None, mode=0, do_pbc=True):
        """CONTACTMAP over contacts (slot i, slot n + i) of pos (2n x 3): (value, deriv
        (2n x 3), virial (n x 3 x 3) for components, (3 x 3) otherwise).  specs: one
        switch definition or one per contact."""
        pos = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(-1, 3))
        n = len(pos) // 2
        specs = [specs] if isinstance(specs, str) else list(specs)
        sws = (_Switch * len(specs))(*[self.switch(sp) for sp in specs])
        ref = np.ascontiguousarray(np.zeros(n) if reference is None else reference, np.float64)
        w = np.ascontiguousarray(np.ones(n) if weight is None else weight, np.float64)
        pb = self.pbc(box)
        nv = n if mode == 0 else 1
        value = np.zeros(nv)
        deriv = np.zeros(6 * n)
        vir = np.zeros(9 * nv)
        self.L.orc_contactmap(C.cast(sws, C.c_void_p), len(specs), n, ref, w, int(mode), C.byref(pb), int(do_pbc),
                              pos.reshape(-1), value, deriv, vir)
        return value, deriv.reshape(2 * n, 3), (vir.reshape(n, 3, 3) if mode == 0 else vir.reshape(3, 3))

    def max_threads(self) -> int:
        return self.L.orc_max_threads()


class Reference:
    """ctypes wrapper of the reference harness (oracle/_ref/libcoord_ref.so)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        self.L = L
        L.ref_switch_eval.argtypes = [C.c_char_p, C.c_int, _dp, C.c_int, _dp, _dp, C.c_char_p, C.c_int]
        L.ref_switch_params.argtypes = [C.c_char_p, _dp]
        L.ref_pbc.argtypes = [_dp, C.c_int, _dp, _dp, _dp, _dp]
        L.ref_linkcells_required.argtypes = [_dp, C.c_double, C.POINTER(C.c_uint * 3), C.c_int,
                                             C.POINTER(C.c_uint * 3), C.POINTER(C.c_uint * 27)]
        L.ref_linkcells_required.restype = C.c_int
        L.ref_nl.argtypes = [C.c_int, C.c_int64, C.c_int64, _dp, _dp, C.c_int, C.c_double, C.c_int, _u32p,
                             C.c_int64]
        L.ref_nl.restype = C.c_int64
        L.ref_coordination.argtypes = [C.c_char_p, C.c_int, C.c_int64, C.c_int64, _i64p, _dp, _dp, C.c_int,
                                       C.c_double, C.c_int, C.c_int, C.POINTER(C.c_double), _dp, _dp]
        L.ref_max_threads.restype = C.c_int

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_SO)

    def switch_eval(self, spec, x, squared=True):
        x = np.ascontiguousarray(x, np.float64)
        f = np.empty_like(x)
        df = np.empty_like(x)
        err = C.create_string_buffer(512)
        if self.L.ref_switch_eval(spec.encode(), len(x), x, int(squared), f, df, err, 512):
            raise ValueError(err.value.decode())
        return f, df

    def switch_params(self, spec):
        out = np.zeros(7)
        if self.L.ref_switch_params(spec.encode(), out):
            raise ValueError(spec)
        return dict(zip(["d0", "dmax", "dmax_2", "invr0", "invr0_2", "stretch", "shift"], out))

    def linkcells_required(self, box, cutoff, cell, use_pbc=True):
        """(cell limits, sorted cells searched from the cell with indices cell)
        by the reference's LinkCells."""
        lim, req = (C.c_uint * 3)(), (C.c_uint * 27)()
        n = self.L.ref_linkcells_required(np.ascontiguousarray(np.asarray(box, np.float64).reshape(9)),
                                          float(cutoff), C.byref((C.c_uint * 3)(*cell)), int(use_pbc), C.byref(lim),
                                          C.byref(req))
        if n < 0:
            raise ValueError("Cell lists cannot be built when passing a box with null volume")
        return list(lim), sorted(req[:n])

    def pbc_distance(self, box, v1, v2):
        v1 = np.ascontiguousarray(np.asarray(v1, np.float64).reshape(-1, 3))
        v2 = np.ascontiguousarray(np.asarray(v2, np.float64).reshape(-1, 3))
        out = np.empty_like(v1)
        inv = np.empty(9)
        self.L.ref_pbc(np.ascontiguousarray(np.asarray(box, np.float64).reshape(9)), len(v1),
                       v1.reshape(-1), v2.reshape(-1), out.reshape(-1), inv)
        return out, inv.reshape(3, 3)

    def nl(self, mode, n0, n1, pos, box, do_pbc, cutoff, cells=False):
        pos = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(-1))
        box = np.ascontiguousarray(np.asarray(box, np.float64).reshape(9))
        cap = max(1024, 64 * (len(pos) // 3))
        while True:
            out = np.empty(2 * cap, np.uint32)
            n = self.L.ref_nl(mode, n0, n1, pos, box, int(do_pbc), float(cutoff), int(cells), out, cap)
            if n < 0:
                raise ValueError("the reference refused the input (an assertion in NeighborList::update)")
            if n <= cap:
                return out[:2 * n].reshape(-1, 2)
            cap = int(n)

    def coordination(self, spec, mode, n0, n1, pos, box, abs_index=None, do_pbc=True, nl_cutoff=0.0,
                     cells=False, nthreads=1):
        pos = np.ascontiguousarray(np.asarray(pos, np.float64).reshape(-1, 3))
        ns = len(pos)
        if abs_index is None:
            abs_index = np.arange(ns, dtype=np.int64)
        abs_index = np.ascontiguousarray(abs_index, dtype=np.int64)
        s = C.c_double()
        deriv = np.zeros(3 * ns)
        vir = np.zeros(9)
        rc = self.L.ref_coordination(spec.encode(), mode, n0, n1, abs_index, pos.reshape(-1),
                                     np.ascontiguousarray(np.asarray(box, np.float64).reshape(9)), int(do_pbc),
                                     float(nl_cutoff), int(cells), int(nthreads), C.byref(s), deriv, vir)
        if rc:
            raise ValueError(spec)
        return s.value, deriv.reshape(ns, 3), vir.reshape(3, 3)

    def max_threads(self) -> int:
        return self.L.ref_max_threads()

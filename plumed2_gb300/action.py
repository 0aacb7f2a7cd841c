"""The COORDINATION action, host side.

``Coordination`` mirrors the reference action's keyword surface and
per-step contract (src/colvar/Coordination.cpp, CoordinationBase.cpp):

    c = Coordination("GROUPA=1-1000 SWITCH={RATIONAL R_0=0.30 NN=6 MM=12 D_MAX=1.0}")
    s, deriv, virial = c.calculate(positions, box, step)

``positions`` are the requested atoms in request order (GROUPA then GROUPB,
as ActionAtomistic::getPositions() returns them), ``box`` is the 3x3 lattice
(rows are lattice vectors, all zero without pbc).  Derivatives and the
virial follow Colvar's layout (Colvar.h:74-113).  Keyword errors raise
``ValueError`` with the reference's messages.  Every number is computed by
libcoordgpu.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import re
from typing import List, Optional, Tuple

import numpy as np

from . import _lib
from ._lib import CoordError, check, dptr

_FLAGS = ("SERIAL", "PAIR", "NLIST", "NLISTCELLS", "NOPBC", "NUMERICAL_DERIVATIVES")
# CoordinationBase::registerKeywords (CoordinationBase.cpp:30-40)
_BASE_KEYS = ("GROUPA", "GROUPB", "NL_CUTOFF", "NL_STRIDE", "LABEL")
# Coordination::registerKeywords (Coordination.cpp:103-115)
_KEYS = _BASE_KEYS + ("SWITCH", "R_0", "NN", "MM", "D_0")


def parse_atom_list(text: str) -> List[int]:
    """GROUPA/GROUPB value: comma-separated serials and ranges a-b or a-b:stride
    (1-based, as Tools::interpretRanges, tools/Tools.cpp:559-601): a range runs
    from a to b inclusive, upwards with a positive stride or downwards with a
    negative one (108-1:-1); any other stride is an error, with the
    reference's message.  Returns 0-based absolute indices."""
    out: List[int] = []
    for tok in text.split(","):
        tok = tok.strip()
        if not tok:
            continue
        m = re.fullmatch(r"(\d+)-(\d+)(?::(-?\d+))?", tok)
        if m:
            a, b, st = int(m.group(1)), int(m.group(2)), int(m.group(3) or 1)
            if (st <= 0) if a <= b else (st >= 0):
                raise ValueError("interpreting ranges %s, stride should be positive" % tok)
            out.extend(i - 1 for i in range(a, b + (1 if a <= b else -1), st))
        elif re.fullmatch(r"\d+", tok):
            out.append(int(tok) - 1)
        else:
            raise ValueError("could not interpret atom list entry '%s'" % tok)
    return out


def split_line(line: str) -> List[str]:
    """Words of an input line; {...} groups stay one word (Tools::getWords)."""
    words, cur, depth = [], "", 0
    for ch in line:
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth -= 1
            if depth < 0:
                raise ValueError("Extra closed parenthesis in '%s'" % line)
        if ch.isspace() and depth == 0:
            if cur:
                words.append(cur)
            cur = ""
        else:
            cur += ch
    if depth != 0:
        raise ValueError("Unmatched parenthesis in '%s'" % line)
    if cur:
        words.append(cur)
    return words


class Coordination:
    """GPU COORDINATION behind the reference's keyword interface."""

    DIRECTIVE = "COORDINATION"
    KEYS = _KEYS

    def __init__(self, line: str = "", *, precision: str = "fp64", device: int = 0, **kw):
        words = split_line(line)
        opts = {}
        flags = set()
        label = None
        for w in words:
            if w.endswith(":") and not opts and not flags and label is None:
                label = w[:-1]
                continue
            if w == self.DIRECTIVE:
                continue
            if "=" in w:
                k, v = w.split("=", 1)
                if v.startswith("{") and v.endswith("}"):
                    v = v[1:-1]
                opts[k.upper()] = v
            else:
                flags.add(w.upper())
        for k, v in kw.items():
            k = k.upper()
            if isinstance(v, bool):
                if v:
                    flags.add(k)
            else:
                opts[k] = v
        self.label = opts.pop("LABEL", label)
        for k in opts:
            if k not in self.KEYS:
                raise ValueError("cannot read keyword %s" % k)
        for f in flags:
            if f not in _FLAGS:
                raise ValueError("cannot read flag %s" % f)
        ga = opts.get("GROUPA", "")
        gb = opts.get("GROUPB", "")
        self.group_a = parse_atom_list(ga) if isinstance(ga, str) else [int(x) for x in ga]
        self.group_b = parse_atom_list(gb) if isinstance(gb, str) else [int(x) for x in gb]
        nlist = "NLIST" in flags
        cells = "NLISTCELLS" in flags
        if nlist and cells:
            raise ValueError("Please activate only one of the two version of the NL")
        self._L = _lib.load()
        p = _lib.CoordParams()
        self._L.coord_params_default(C.byref(p))
        self._switch_bytes = None
        self._set_switch(p, opts)
        p.nopbc = int("NOPBC" in flags)
        p.pair = int("PAIR" in flags)
        p.serial = int("SERIAL" in flags)
        p.nlist = _lib.NL_CLASSIC if nlist else (_lib.NL_CELLS if cells else _lib.NL_NONE)
        p.nl_cutoff = float(opts.get("NL_CUTOFF", 0.0))
        p.nl_stride = int(float(opts.get("NL_STRIDE", 0)))
        p.precision = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[precision]
        p.device = device
        self.params = p
        self.precision = precision
        ctx = C.c_void_p()
        rc = self._L.coord_create(C.byref(p), C.byref(ctx))
        self._ctx = ctx
        if rc != 0:
            msg = self._L.coord_last_error(ctx).decode() if ctx.value else ""
            self.close()
            raise ValueError(msg) if rc == _lib.COORD_ERR_ARG else CoordError(rc, msg)
        self._groups_set = False
        try:
            self._configure(opts)
        except Exception:
            self.close()
            raise

    def _set_switch(self, p, opts):
        """SWITCH or R_0/NN/MM/D_0 (Coordination.cpp:128-157)."""
        sw = opts.get("SWITCH", "")
        self._switch_bytes = sw.encode() if sw else None
        p.switch_def = self._switch_bytes
        if not sw:
            p.r0 = float(opts.get("R_0", 0.0))
            p.d0 = float(opts.get("D_0", 0.0))
            p.nn = int(opts.get("NN", 6))
            p.mm = int(opts.get("MM", 0))

    def _configure(self, opts):
        """Set-up after coord_create (the sibling CVs' own keywords)."""

    def _status(self, rc):
        if rc == _lib.COORD_ERR_ARG:
            raise ValueError(self._L.coord_last_error(self._ctx).decode())
        check(self._L, self._ctx, rc)

    # -- groups ------------------------------------------------------------
    def _ensure_groups(self):
        if self._groups_set:
            return
        a = np.ascontiguousarray(self.group_a, dtype=np.int64)
        b = np.ascontiguousarray(self.group_b, dtype=np.int64)
        rc = self._L.coord_set_groups(self._ctx, a.ctypes.data_as(C.POINTER(C.c_int64)), len(a),
                                      b.ctypes.data_as(C.POINTER(C.c_int64)), len(b))
        if rc == _lib.COORD_ERR_ARG:
            raise ValueError(self._L.coord_last_error(self._ctx).decode())
        check(self._L, self._ctx, rc)
        self._groups_set = True

    @property
    def nslots(self) -> int:
        return len(self.group_a) + len(self.group_b)

    @property
    def requested_atoms(self) -> List[int]:
        """Absolute atom indices in request order (CoordinationBase.cpp:99)."""
        return list(self.group_a) + list(self.group_b)

    # -- per step ----------------------------------------------------------
    def calculate(self, positions, box, step: int = 0, rebuild: bool = False, derivatives: bool = True,
                  out=None) -> Tuple[float, Optional[np.ndarray], Optional[np.ndarray]]:
        """One step through the host-buffer call (coord_forward).  out=(deriv (nslots, 3), virial (9,)) reuses
        the caller's float64 C-contiguous arrays, as an MD engine reuses its force arrays from step to step."""
        self._ensure_groups()
        pos = np.ascontiguousarray(np.asarray(positions, dtype=np.float64).reshape(-1, 3))
        if len(pos) != self.nslots:
            raise ValueError("expected %d positions, got %d" % (self.nslots, len(pos)))
        bx = np.ascontiguousarray(np.asarray(box, dtype=np.float64).reshape(9))
        s = C.c_double()
        if out is not None and derivatives:
            deriv, vir = out
            if (deriv.dtype != np.float64 or not deriv.flags.c_contiguous or deriv.size != 3 * self.nslots or
                    vir.dtype != np.float64 or not vir.flags.c_contiguous or vir.size != 9):
                raise ValueError("out needs float64 C-contiguous arrays of %d and 9 values" % (3 * self.nslots))
        else:
            deriv = np.zeros((self.nslots, 3)) if derivatives else None
            vir = np.zeros(9) if derivatives else None
        flags = (_lib.FLAG_REBUILD if rebuild else 0) | (0 if derivatives else _lib.FLAG_NO_DERIV)
        rc = self._L.coord_forward(self._ctx, dptr(pos), dptr(bx), int(step), flags, C.byref(s),
                                   dptr(deriv) if derivatives else None, dptr(vir) if derivatives else None)
        check(self._L, self._ctx, rc)
        return s.value, deriv, (vir.reshape(3, 3) if derivatives else None)

    def forward_host(self, pos_addr: int, box_addr: int, step: int, flags: int, s_addr: int, deriv_addr: int,
                     virial_addr: int):
        """coord_forward with plain addresses of host arrays (positions nslots x 3, box 9, s 1, derivatives
        nslots x 3, virial 9): the call a compiled caller such as the PLUMED plugin makes, with no array
        checks on the Python side."""
        self._ensure_groups()
        rc = self._L.coord_forward_addr(self._ctx, pos_addr, box_addr, int(step), int(flags), s_addr,
                                        deriv_addr or None, virial_addr or None)
        if rc:
            check(self._L, self._ctx, rc)

    def forward_host_batch(self, n_frames: int, pos_addr: int, boxes_addr: int, step: int, flags: int, s_addr: int,
                           deriv_addr: int, virial_addr: int):
        """coord_forward_batch with plain addresses of host arrays: positions
        [frames][slots][3], boxes [frames][9], s [frames], derivatives
        [frames][slots][3], virial [frames][9]."""
        self._ensure_groups()
        rc = self._L.coord_forward_batch(self._ctx, int(n_frames), pos_addr, boxes_addr, int(step), int(flags), s_addr,
                                         deriv_addr or None, virial_addr or None)
        if rc:
            check(self._L, self._ctx, rc)

    def calculate_system(self, system_positions, box, step: int = 0, **kw):
        """Gather the requested atoms from a full system array and calculate."""
        sp = np.asarray(system_positions, dtype=np.float64).reshape(-1, 3)
        return self.calculate(sp[self.requested_atoms], box, step, **kw)

    def forward_device(self, pos_ptr: int, boxes, n_frames: int, s_ptr: int, deriv_ptr: int = 0,
                       virial_ptr: int = 0, step: int = 0, flags: int = 0, stream: int = 0, dparam_ptr: int = 0):
        """Device-pointer batched forward (pointers as integers, e.g. tensor.data_ptr())."""
        self._ensure_groups()
        bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(-1, 9))
        if len(bx) != n_frames:
            raise ValueError("need one box per frame")
        rc = self._L.coord_forward_device(self._ctx, int(n_frames), C.c_void_p(pos_ptr), dptr(bx), int(step),
                                          int(flags), C.c_void_p(s_ptr), C.c_void_p(deriv_ptr or None),
                                          C.c_void_p(virial_ptr or None), C.c_void_p(dparam_ptr or None),
                                          C.c_void_p(stream or None))
        check(self._L, self._ctx, rc)

    def backward_device(self, pos_ptr: int, boxes, n_frames: int, g_ptr: int, grad_pos_ptr: int = 0,
                        grad_box_ptr: int = 0, grad_param_ptr: int = 0, stream: int = 0):
        self._ensure_groups()
        bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(-1, 9))
        rc = self._L.coord_backward_device(self._ctx, int(n_frames), C.c_void_p(pos_ptr), dptr(bx),
                                           C.c_void_p(g_ptr), C.c_void_p(grad_pos_ptr or None),
                                           C.c_void_p(grad_box_ptr or None), C.c_void_p(grad_param_ptr or None),
                                           C.c_void_p(stream or None))
        check(self._L, self._ctx, rc)

    def apply_forces(self, n_frames: int, ff_ptr: int, n_atoms: int, atom_forces_ptr: int = 0, box_forces_ptr: int = 0,
                     stream: int = 0):
        """coord_apply_forces: ff (force on the CV, -dV/ds, per frame) times the saved ds/dx added into the
        engine's [n_frames][n_atoms][3] force array by absolute index, and times the virial into the box
        force (device pointers)."""
        self._ensure_groups()
        rc = self._L.coord_apply_forces(self._ctx, int(n_frames), C.c_void_p(ff_ptr), int(n_atoms),
                                        C.c_void_p(atom_forces_ptr or None), C.c_void_p(box_forces_ptr or None),
                                        C.c_void_p(stream or None))
        check(self._L, self._ctx, rc)

    # -- neighbour list ------------------------------------------------------
    def nl_size(self, frame: int = 0) -> int:
        n = C.c_int64()
        check(self._L, self._ctx, self._L.coord_nl_size(self._ctx, frame, C.byref(n)))
        return n.value

    # how the last host-array call moved the arrays (coord_host_path)
    HOST_PATHS = {-1: None, 0: "staged", 1: "direct", 2: "chunked"}

    def host_path(self):
        """'staged', 'direct' or 'chunked' for the last forward_host / forward_host_batch, or None."""
        return self.HOST_PATHS.get(self._L.coord_host_path(self._ctx))

    def nl_near_size(self, frame: int = 0):
        """(entries in the rows' near parts, skin): coord_nl_near_size."""
        n, sk = C.c_int64(), C.c_double()
        check(self._L, self._ctx, self._L.coord_nl_near_size(self._ctx, frame, C.byref(n), C.byref(sk)))
        return n.value, sk.value

    def pairs(self, frame: int = 0) -> np.ndarray:
        n = C.c_int64()
        check(self._L, self._ctx, self._L.coord_get_pairs(self._ctx, frame, None, 0, C.byref(n)))
        out = np.zeros(2 * max(n.value, 1), dtype=np.uint32)
        check(self._L, self._ctx, self._L.coord_get_pairs(self._ctx, frame, out.ctypes.data_as(
            C.POINTER(C.c_uint32)), n.value, C.byref(n)))
        return out[:2 * n.value].reshape(-1, 2)

    # -- switching function ------------------------------------------------
    def switch(self, x, squared: bool = True):
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = np.empty_like(x)
        df = np.empty_like(x)
        check(self._L, self._ctx, self._L.coord_switch_eval(self._ctx, len(x), dptr(x), int(squared), dptr(f),
                                                             dptr(df)))
        return f, df

    def switch_params(self) -> dict:
        out = np.zeros(7)
        check(self._L, self._ctx, self._L.coord_switch_params(self._ctx, dptr(out)))
        return dict(zip(["d0", "dmax", "dmax_2", "invr0", "invr0_2", "stretch", "shift"], out))

    # -- tuning / timing -----------------------------------------------------
    def set_timing(self, enable: bool = True):
        check(self._L, self._ctx, self._L.coord_set_timing(self._ctx, int(enable)))

    def kernel_times(self):
        """Per-launch device times (ms) of the pair kernel since timing was enabled/last read."""
        n = C.c_int()
        check(self._L, self._ctx, self._L.coord_kernel_times(self._ctx, None, 0, C.byref(n)))
        out = (C.c_float * max(n.value, 1))()
        check(self._L, self._ctx, self._L.coord_kernel_times(self._ctx, out, n.value, C.byref(n)))
        return list(out)[:n.value]

    def kernel_ms(self):
        """(average ms, launches) of the pair kernel since timing was enabled/last read."""
        ms = C.c_double()
        n = C.c_int()
        check(self._L, self._ctx, self._L.coord_last_kernel_ms(self._ctx, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def autotune(self) -> str:
        buf = C.create_string_buffer(256)
        check(self._L, self._ctx, self._L.coord_autotune(self._ctx, buf, 256))
        return buf.value.decode()

    def close(self):
        if getattr(self, "_ctx", None) is not None and self._ctx.value:
            self._L.coord_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DHEnergy(Coordination):
    """DHENERGY (colvar/DHEnergy.cpp:62): Debye-Hueckel energy between GROUPA and
    GROUPB (or within GROUPA) with CoordinationBase's loop and keywords, plus
    I (1.0 M), TEMP (300.0 K), EPSILON (80.0).  ``charges`` are the atoms'
    charges by absolute atom index (Atoms::getCharge), ``units`` the action's
    (energy, length, charge) units in kJ/mol, nm, e.  FP64 only."""

    DIRECTIVE = "DHENERGY"
    KEYS = _BASE_KEYS + ("I", "TEMP", "EPSILON")

    def __init__(self, line: str = "", *, charges=None, units=(1.0, 1.0, 1.0), device: int = 0, **kw):
        self._charges = charges
        self._units = tuple(float(u) for u in units)
        super().__init__(line, precision="fp64", device=device, **kw)

    def _set_switch(self, p, opts):
        p.r0 = 1.0  # the switching function is not used by this CV

    def _configure(self, opts):
        ionic = float(opts.get("I", 1.0))
        temp = float(opts.get("TEMP", 300.0))
        eps = float(opts.get("EPSILON", 80.0))
        self.ionic, self.temp, self.epsilon = ionic, temp, eps
        self._status(self._L.coord_set_dhenergy(self._ctx, ionic, temp, eps, *self._units))
        if self._charges is not None:
            self.set_charges(self._charges)

    def set_charges(self, charges):
        """Charges by absolute atom index, covering every atom of the groups."""
        q = np.ascontiguousarray(charges, dtype=np.float64).reshape(-1)
        self._status(self._L.coord_set_charges(self._ctx, dptr(q), len(q)))


class GHBFIX(Coordination):
    """GHBFIX (colvar/GHBFIX.cpp:63): the generalised hydrogen-bond fix energy
    with CoordinationBase's loop and keywords, plus D_0, D_MAX, C (compulsory),
    TYPES and PARAMS (table files, compulsory) and ENERGY_UNITS.  The tables
    may be given as text (``types_text``/``params_text``) instead of files;
    ``plumed_energy`` is the action's energy unit in kJ/mol.  FP64 only."""

    DIRECTIVE = "GHBFIX"
    KEYS = _BASE_KEYS + ("D_0", "D_MAX", "C", "TYPES", "PARAMS", "ENERGY_UNITS")

    def __init__(self, line: str = "", *, types_text: Optional[str] = None, params_text: Optional[str] = None,
                 plumed_energy: float = 1.0, device: int = 0, **kw):
        self._texts = (types_text, params_text)
        self._plumed_energy = float(plumed_energy)
        super().__init__(line, precision="fp64", device=device, **kw)

    def _set_switch(self, p, opts):
        p.r0 = 1.0  # the switching function is not used by this CV

    def _configure(self, opts):
        from .siblings import ghbfix_tables
        for k in ("D_0", "D_MAX", "C"):
            if k not in opts:
                raise ValueError("keyword %s is compulsory for this action" % k)
        types_text, params_text = self._texts
        if types_text is None or params_text is None:
            for k in ("TYPES", "PARAMS"):
                if k not in opts:
                    raise ValueError("keyword %s is compulsory for this action" % k)
            with open(opts["TYPES"]) as f:
                types_text = f.read()
            with open(opts["PARAMS"]) as f:
                params_text = f.read()
        types, eta = ghbfix_tables(types_text, params_text, opts.get("ENERGY_UNITS", "plumed"), self._plumed_energy)
        self.types, self.eta = types, eta
        d0, dmax, cc = float(opts["D_0"]), float(opts["D_MAX"]), float(opts["C"])
        t = np.ascontiguousarray(types, dtype=np.int32)
        e = np.ascontiguousarray(eta, dtype=np.float64).reshape(-1)
        self._status(self._L.coord_set_ghbfix(self._ctx, d0, dmax, cc, t.ctypes.data_as(C.POINTER(C.c_int32)),
                                              len(t), dptr(e), eta.shape[0]))


class CoordinationNumbers:
    """COORDINATIONNUMBER (symfunc/CoordinationNumbers.cpp:247-309): per-atom
    coordination numbers cn_i = sum_j sigma(r_ij), the reference's
    CONTACT_MATRIX (adjmat/ContactMatrix.h) times a vector of ones, on the GPU.

        c = CoordinationNumbers("SPECIES=1-400 SWITCH={RATIONAL D_0=3.0 R_0=1.5 D_MAX=6.0}")
        cn = c.calculate(positions, box)          # one value per SPECIES atom

    Keywords: SPECIES, or SPECIESA with SPECIESB; SWITCH or R_0/NN/MM/D_0.  The
    contact matrix's link cells have cutoff d_max, so the pairs are a
    neighbour list with NL_CUTOFF = d_max rebuilt every call (the same
    inclusive test).  A switch without D_MAX weighs every pair: the list
    cutoff then covers every minimum-image distance of the box.  Positions
    are the requested atoms in request order (SPECIES, or SPECIESA then
    SPECIESB); the box is periodic."""

    KEYS = ("SPECIES", "SPECIESA", "SPECIESB", "SWITCH", "R_0", "NN", "MM", "D_0", "LABEL")

    def __init__(self, line: str = "", *, precision: str = "fp64", device: int = 0):
        words = split_line(line)
        opts = {}
        for w in words:
            if w.endswith(":") and not opts:
                opts["LABEL"] = w[:-1]
                continue
            if w == "COORDINATIONNUMBER":
                continue
            if "=" not in w:
                raise ValueError("cannot read flag %s" % w)
            k, v = w.split("=", 1)
            if v.startswith("{") and v.endswith("}"):
                v = v[1:-1]
            if k.upper() not in self.KEYS:
                raise ValueError("cannot read keyword %s" % k)
            opts[k.upper()] = v
        if "SPECIES" in opts:
            self.group_a, self.group_b = parse_atom_list(opts["SPECIES"]), []
        elif "SPECIESA" in opts and "SPECIESB" in opts:
            self.group_a, self.group_b = parse_atom_list(opts["SPECIESA"]), parse_atom_list(opts["SPECIESB"])
        else:
            raise ValueError("missing atoms input use SPECIES or SPECIESA/SPECIESB")
        if "SWITCH" in opts:
            self._switch = "SWITCH={%s}" % opts["SWITCH"]
        elif "R_0" in opts:
            self._switch = " ".join("%s=%s" % (k, opts[k]) for k in ("R_0", "NN", "MM", "D_0") if k in opts)
        else:
            raise ValueError("missing switching function parameters use SWITCH/R_0")
        self.precision, self.device = precision, device
        self._act = None
        self._cut = None
        # d_max of the switch (huge without D_MAX)
        probe = Coordination("GROUPA=1 " + self._switch, precision="fp64", device=device)
        self.dmax = probe.switch_params()["dmax"]
        probe.close()

    @property
    def nslots(self) -> int:
        return len(self.group_a) + len(self.group_b)

    def _action(self, boxes):
        """The Coordination context whose list holds the contact matrix's pairs."""
        b = np.asarray(boxes, dtype=np.float64).reshape(-1, 3, 3)
        reach = 0.5 * np.linalg.norm(b, axis=2).sum(axis=1).max() * (1.0 + 1e-9) + 1e-9
        cut = self.dmax if self.dmax < reach else reach
        if self._act is None or (self._cut < reach and cut != self._cut):
            if self._act is not None:
                self._act.close()
            ga = ",".join(str(i + 1) for i in self.group_a)
            gb = ",".join(str(i + 1) for i in self.group_b)
            line = "GROUPA=%s%s %s NLIST NL_CUTOFF=%.17g NL_STRIDE=1" % (ga, " GROUPB=" + gb if gb else "",
                                                                        self._switch, cut)
            self._act = Coordination(line, precision=self.precision, device=self.device)
            self._act._ensure_groups()
            self._cut = cut
        return self._act

    def forward_device(self, pos_ptr: int, boxes, n_frames: int, cn_ptr: int, s_ptr: int = 0, stream: int = 0,
                       step: int = 0):
        """cn [frames][slots] (device) for device positions [frames][slots][3]."""
        act = self._action(boxes)
        bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(-1, 9))
        rc = act._L.coord_peratom_device(act._ctx, int(n_frames), C.c_void_p(pos_ptr), dptr(bx), int(step), 0,
                                         C.c_void_p(cn_ptr), C.c_void_p(s_ptr or None), C.c_void_p(stream or None))
        check(act._L, act._ctx, rc)

    def backward_device(self, pos_ptr: int, boxes, n_frames: int, g_ptr: int, grad_pos_ptr: int,
                        grad_box_ptr: int = 0, stream: int = 0):
        """dV/dx [frames][slots][3] and dV/dh [frames][9] for dV/dcn = g [frames][slots]."""
        act = self._action(boxes)
        bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(-1, 9))
        rc = act._L.coord_peratom_backward_device(act._ctx, int(n_frames), C.c_void_p(pos_ptr), dptr(bx),
                                                  C.c_void_p(g_ptr), C.c_void_p(grad_pos_ptr),
                                                  C.c_void_p(grad_box_ptr or None), C.c_void_p(stream or None))
        check(act._L, act._ctx, rc)

    def calculate(self, positions, box, step: int = 0, all_slots: bool = False) -> np.ndarray:
        """cn of the SPECIES (or SPECIESA) atoms; all_slots: also the SPECIESB
        column sums."""
        import torch
        pos = torch.as_tensor(np.ascontiguousarray(np.asarray(positions, np.float64).reshape(1, -1, 3)),
                              device="cuda:%d" % self.device)
        if pos.shape[1] != self.nslots:
            raise ValueError("expected %d positions, got %d" % (self.nslots, pos.shape[1]))
        cn = torch.empty(1, self.nslots, dtype=torch.float64, device=pos.device)
        self.forward_device(pos.data_ptr(), np.asarray(box, np.float64).reshape(1, 9), 1, cn.data_ptr(), step=step)
        out = cn[0].cpu().numpy()
        return out if all_slots else out[:len(self.group_a)]

    def close(self):
        if self._act is not None:
            self._act.close()
            self._act = None


class ContactMap:
    """CONTACTMAP (colvar/ContactMap.cpp:149-365) on the GPU.

        cm = ContactMap("ATOMS1=1,2 ATOMS2=5,9 SWITCH={RATIONAL R_0=0.5} SUM")
        value, deriv, virial = cm.calculate(positions, box)

    Keywords as the reference reads them: ATOMSn (two atoms each, numbered
    from 1 until one is missing); SWITCHn for every contact, or one SWITCH;
    REFERENCEn or REFERENCE (default 0); WEIGHTn or WEIGHT (default 1); flags
    SUM, CMDIST (not both), NOPBC, SERIAL.  positions are the requested atoms:
    the first atoms of all contacts, then the second atoms.  Without SUM or
    CMDIST, value holds one component per contact (contact-n) and virial one
    box derivative per contact."""

    FLAGS = ("SUM", "CMDIST", "NOPBC", "SERIAL")

    def __init__(self, line: str = "", *, device: int = 0):
        opts, flags = {}, set()
        for w in split_line(line):
            if w.endswith(":") and not opts and not flags:
                opts["LABEL"] = w[:-1]
                continue
            if w == "CONTACTMAP":
                continue
            if "=" in w:
                k, v = w.split("=", 1)
                if v.startswith("{") and v.endswith("}"):
                    v = v[1:-1]
                opts[k.upper()] = v
            else:
                if w.upper() not in self.FLAGS:
                    raise ValueError("cannot read flag %s" % w)
                flags.add(w.upper())
        self.label = opts.pop("LABEL", None)
        dosum, docmdist = "SUM" in flags, "CMDIST" in flags
        if dosum and docmdist:
            raise ValueError("You cannot use SUM and CMDIST together")
        first, second = [], []
        i = 1
        while "ATOMS%d" % i in opts:
            at = parse_atom_list(opts.pop("ATOMS%d" % i))
            if len(at) != 2:
                raise ValueError("ATOMS%d keyword has the wrong number of atoms" % i)
            first.append(at[0])
            second.append(at[1])
            i += 1
        n = len(first)
        if n == 0:
            raise ValueError("no contacts: use ATOMS1, ATOMS2, ...")
        sws = []
        for i in range(1, n + 1):
            if "SWITCH%d" % i not in opts:
                break
            sws.append(opts.pop("SWITCH%d" % i))
        if not sws:
            if "SWITCH" not in opts:
                raise ValueError("no switching function specified use SWITCH keyword")
            sws = [opts.pop("SWITCH")]
        elif len(sws) != n:
            raise ValueError("missing SWITCH%d keyword" % (len(sws) + 1))
        ref = np.zeros(n)
        counted = 0
        for i in range(1, n + 1):
            if "REFERENCE%d" % i not in opts:
                break
            ref[i - 1] = float(opts.pop("REFERENCE%d" % i))
            counted += 1
        if counted == 0:
            ref[:] = float(opts.pop("REFERENCE", 0.0))
            counted = n - 1  # the reference copies REFERENCE into contacts 2..n
        if counted == 0 and docmdist:
            raise ValueError("with CMDIST one must use REFERENCE to setup the reference contact map")
        w = np.ones(n)
        counted = 0
        for i in range(1, n + 1):
            if "WEIGHT%d" % i not in opts:
                break
            w[i - 1] = float(opts.pop("WEIGHT%d" % i))
            counted += 1
        if counted == 0:
            w[:] = float(opts.pop("WEIGHT", 1.0))
        for k in opts:
            raise ValueError("cannot read keyword %s" % k)
        self.first, self.second = first, second
        self.n = n
        self.mode = _lib.CMAP_CMDIST if docmdist else (_lib.CMAP_SUM if dosum else _lib.CMAP_COMPONENTS)
        self.reference, self.weight = ref, w
        self.switches = sws
        self.device = device
        self._L = _lib.load()
        self._m = C.c_void_p()
        defs = (C.c_char_p * len(sws))(*[s.encode() for s in sws])
        rc = self._L.coord_cmap_create(n, defs, len(sws), dptr(ref), dptr(w), self.mode, int("NOPBC" in flags), device,
                                       C.byref(self._m))
        if rc:
            msg = self._L.coord_cmap_last_error(self._m).decode()
            self.close()
            raise ValueError(msg) if rc == _lib.COORD_ERR_ARG else CoordError(rc, msg)

    @property
    def requested_atoms(self) -> List[int]:
        return list(self.first) + list(self.second)

    def forward_device(self, pos_ptr: int, boxes, n_frames: int, value_ptr: int, deriv_ptr: int = 0,
                       virial_ptr: int = 0, stream: int = 0):
        bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(-1, 9))
        rc = self._L.coord_cmap_forward_device(self._m, int(n_frames), C.c_void_p(pos_ptr), dptr(bx),
                                               C.c_void_p(value_ptr), C.c_void_p(deriv_ptr or None),
                                               C.c_void_p(virial_ptr or None), C.c_void_p(stream or None))
        if rc:
            raise CoordError(rc, self._L.coord_cmap_last_error(self._m).decode())

    def calculate(self, positions, box):
        """(value, deriv (2n x 3), virial): value and virial per contact
        without SUM/CMDIST ((n,), (n, 3, 3)), else a float and (3, 3)."""
        import torch
        dev = "cuda:%d" % self.device
        pos = torch.as_tensor(np.ascontiguousarray(np.asarray(positions, np.float64).reshape(1, -1, 3)), device=dev)
        if pos.shape[1] != 2 * self.n:
            raise ValueError("expected %d positions, got %d" % (2 * self.n, pos.shape[1]))
        nv = self.n if self.mode == _lib.CMAP_COMPONENTS else 1
        value = torch.empty(nv, dtype=torch.float64, device=dev)
        deriv = torch.empty(2 * self.n, 3, dtype=torch.float64, device=dev)
        vir = torch.empty(nv, 9, dtype=torch.float64, device=dev)
        self.forward_device(pos.data_ptr(), np.asarray(box, np.float64).reshape(1, 9), 1, value.data_ptr(),
                            deriv.data_ptr(), vir.data_ptr())
        v, d, w = value.cpu().numpy(), deriv.cpu().numpy(), vir.cpu().numpy().reshape(nv, 3, 3)
        if self.mode == _lib.CMAP_COMPONENTS:
            return v, d, w
        return float(v[0]), d, w[0]

    def close(self):
        if getattr(self, "_m", None) is not None and self._m.value:
            self._L.coord_cmap_destroy(self._m)
            self._m = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

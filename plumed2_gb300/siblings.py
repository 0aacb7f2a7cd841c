"""Host-side set-up of the sibling CVs of CoordinationBase: DHENERGY and GHBFIX.

Both reuse COORDINATION's pair loop with another ``pairing()``; what differs
is read here, on the host, exactly as the reference's constructors read it:

* DHENERGY (colvar/DHEnergy.cpp:80-114): keywords I (1.0), TEMP (300.0),
  EPSILON (80.0); per-atom charges come from the MD engine.
* GHBFIX (colvar/GHBFIX.cpp:80-171): keywords D_0, D_MAX, C, TYPES, PARAMS,
  ENERGY_UNITS; TYPES and PARAMS are PLUMED-format tables (``#! FIELDS``).
"""
from __future__ import annotations

import numpy as np

# Units::setEnergy(const std::string&) (tools/Units.cpp:40-60)
ENERGY_UNITS = {"kj/mol": 1.0, "kcal/mol": 4.184, "j/mol": 0.001, "eV": 96.48530749925792, "Ha": 2625.499638}


def energy_unit(name: str) -> float:
    """The energy unit in kJ/mol for a unit name or a number, as Units::setEnergy."""
    if name in ENERGY_UNITS:
        return ENERGY_UNITS[name]
    try:
        v = float(name)
    except ValueError:
        raise ValueError("problem with setting the energy unit, either use give an numerical value or use one of "
                         "the defined units: kj/mol, kcal/mol, j/mol, eV, Ha (case sensitive)") from None
    if not v > 0.0:
        raise ValueError("energy unit should be positive")
    return v


def table_rows(text: str, fields):
    """Rows of a PLUMED table (IFile): a ``#! FIELDS`` line names the columns,
    other ``#`` lines and blank lines are skipped; each row is returned as a
    dict of the requested fields."""
    names = None
    out = []
    for line in text.splitlines():
        s = line.strip()
        if not s:
            continue
        if s.startswith("#!"):
            w = s[2:].split()
            if w and w[0] == "FIELDS":
                names = w[1:]
            continue
        if s.startswith("#"):
            continue
        if names is None:
            raise ValueError("table without a #! FIELDS line")
        vals = s.split()
        if len(vals) < len(names):
            raise ValueError("table row with %d fields, %d named: %r" % (len(vals), len(names), line))
        row = dict(zip(names, vals))
        missing = [f for f in fields if f not in row]
        if missing:
            raise ValueError("table has no field %s" % missing[0])
        out.append({f: row[f] for f in fields})
    return out


def ghbfix_tables(types_text: str, params_text: str, energy_units: str = "plumed", plumed_energy: float = 1.0):
    """(types, eta) of GHBFIX::GHBFIX (GHBFIX.cpp:131-170).

    types[a] is the type id of absolute atom a: ids in order of first
    appearance in TYPES.  eta is the n x n scaling matrix, eta[n*t1+t2] from
    PARAMS.  A type name in PARAMS that TYPES never named maps to id 0, as the
    reference's std::map::operator[] lookup inserts it with value 0.  With
    ENERGY_UNITS other than "plumed" eta is converted to the plumed energy unit
    (plumed_energy, in kJ/mol)."""
    ids = {}
    types = []
    for row in table_rows(types_text, ["itype"]):
        it = row["itype"]
        if not it:
            raise ValueError("itype is empty")
        if it not in ids:
            ids[it] = len(ids)  # 0 first, then the largest id so far + 1
        types.append(ids[it])
    if not types:
        raise ValueError("empty TYPES table")
    n = max(types) + 1
    eta = np.zeros(n * n)
    for row in table_rows(params_text, ["itype", "jtype", "eta"]):
        ti = ids.setdefault(row["itype"], 0)
        tj = ids.setdefault(row["jtype"], 0)
        eta[n * ti + tj] = float(row["eta"])
    if energy_units != "plumed":
        eta = eta * (energy_unit(energy_units) / plumed_energy)
    return np.asarray(types, np.int32), eta.reshape(n, n)

"""Mesh and boundary-condition files in the reference's CSV format (ImportFromCSV.h:23-253).

Each file has one header line, then records.  The reference reads the records with
``ifs >> buf`` (whitespace-separated tokens) and splits every token on ',' with
``std::getline``; the first field is an id and the rest are values, parsed with
``std::stod`` / ``std::stoi``.  These readers follow that grammar exactly, so a file the
reference accepts gives the same lists here, in the same order:

* a record is a whitespace-free token, not a line (``"0, 1"`` is two records);
* a token whose first field is empty is skipped;
* the node id of Node.csv and the element id of Element.csv are not used: nodes and
  elements are numbered by their position in the file;
* in Dirichlet.csv and Neumann.csv the value fields are the dofs 0, 1, 2, ... in order, and
  ``free`` leaves that dof out;
* numbers are parsed as the C library parses them (the longest valid prefix); an empty or
  non-numeric field raises ValueError and a value out of range (overflow, or underflow to a
  subnormal) OverflowError, where ``std::stod`` / ``std::stoi`` throw.

A file that cannot be opened raises OSError with the reference's message.
"""
import ctypes as C
import ctypes.util
import errno

import numpy as np

_libc = C.CDLL(ctypes.util.find_library("c") or None, use_errno=True)
_libc.strtod.restype = C.c_double
_libc.strtod.argtypes = [C.c_char_p, C.POINTER(C.c_char_p)]
_libc.strtol.restype = C.c_long
_libc.strtol.argtypes = [C.c_char_p, C.POINTER(C.c_char_p), C.c_int]


def _stod_prefix(s):
    """std::stod: the value strtod gives for the field, ValueError when it converts nothing."""
    buf = C.create_string_buffer(s)
    end = C.c_char_p()
    C.set_errno(0)
    v = _libc.strtod(buf, C.byref(end))
    err = C.get_errno()
    used = C.cast(end, C.c_void_p).value - C.addressof(buf)
    if used == 0:
        raise ValueError(f"stod: no conversion of {s!r}")
    if err == errno.ERANGE:   # std::out_of_range, also for results that underflow
        raise OverflowError(f"stod: {s!r} out of range")
    return float(v)


def _stoi(s):
    """std::stoi: strtol base 10 on the field, within int range."""
    buf = C.create_string_buffer(s)
    end = C.c_char_p()
    C.set_errno(0)
    v = _libc.strtol(buf, C.byref(end), 10)
    err = C.get_errno()
    used = C.cast(end, C.c_void_p).value - C.addressof(buf)
    if used == 0:
        raise ValueError(f"stoi: no conversion of {s!r}")
    if err == errno.ERANGE or not -2**31 <= v < 2**31:
        raise OverflowError(f"stoi: {s!r} out of range")
    return int(v)


class _Fields:
    """std::getline(stream, str, ',') over one token, with the stream's eof/fail states: a
    read after the end leaves str unchanged, as the sentry refuses it."""

    def __init__(self, token):
        self.t, self.pos, self.eof, self.fail, self.str = token, 0, False, False, b""

    def next(self):
        if self.fail or self.eof:
            self.fail = True
            return False
        self.str = b""
        k = self.t.find(b",", self.pos)
        if k < 0:
            self.str = self.t[self.pos:]
            self.pos = len(self.t)
            self.eof = True
            if not self.str:
                self.fail = True
                return False
            return True
        self.str = self.t[self.pos:k]
        self.pos = k + 1
        return True


def _records(fname, what):
    try:
        with open(fname, "rb") as fh:
            text = fh.read()
    except OSError as e:
        raise OSError(f"{what} file {fname} open error!") from e
    nl = text.find(b"\n")
    body = b"" if nl < 0 else text[nl + 1:]
    for token in body.split():   # bytes.split: the C locale's whitespace, as operator>>
        f = _Fields(token)
        f.next()
        if f.str:
            yield f


def import_nodes_from_csv(fname):
    """ImportNodesFromCSV (ImportFromCSV.h:22-58): coordinates, one row per node.  Rows of
    different lengths come back as a list of arrays."""
    rows = []
    for f in _records(fname, "Node"):
        x = []
        while f.next():
            x.append(_stod_prefix(f.str))
        rows.append(x)
    if rows and all(len(r) == len(rows[0]) for r in rows):
        return np.array(rows, dtype=float).reshape(len(rows), len(rows[0]))
    return [np.array(r, dtype=float) for r in rows]


def import_elements_from_csv(fname):
    """ImportElementsFromCSV (ImportFromCSV.h:63-98): node ids of each element."""
    rows = []
    for f in _records(fname, "Element"):
        el = []
        while f.next():
            el.append(_stoi(f.str))
        rows.append(el)
    if rows and all(len(r) == len(rows[0]) for r in rows):
        return np.array(rows, dtype=np.int32).reshape(len(rows), len(rows[0]))
    return [np.array(r, dtype=np.int32) for r in rows]


def _conditions(fname, what):
    out = []
    for f in _records(fname, what):
        idn = _stoi(f.str)
        i = 0
        while f.next():
            if f.str != b"free":
                out.append(((idn, i), _stod_prefix(f.str)))
            i += 1
    return out


def import_dirichlet_from_csv(fname):
    """ImportDirichletFromCSV (ImportFromCSV.h:103-137): [((node, dof), value), ...]."""
    return _conditions(fname, "Dirichlet Condition")


def import_neumann_from_csv(fname):
    """ImportNeumannFromCSV (ImportFromCSV.h:142-176): [((node, dof), value), ...].  The
    reference prints the Dirichlet message for this file too (ImportFromCSV.h:147)."""
    return _conditions(fname, "Dirichlet Condition")


def import_initial_from_csv(u, fname):
    """ImportInitialFromCSV (ImportFromCSV.h:181-216): sets u[node, dof] in place for the
    fields that are not ``free``; u is (nnodes, ndof)."""
    for f in _records(fname, "Initial Condition"):
        idn = _stoi(f.str)
        for i in range(u.shape[1]):
            f.next()
            if f.str != b"free":
                u[idn, i] = _stod_prefix(f.str)
    return u


def import_periodic_from_csv(fname):
    """ImportPeriodicFromCSV (ImportFromCSV.h:221-253): [(master, slave), ...]."""
    out = []
    for f in _records(fname, "Periodic Boundary Condition"):
        master = _stoi(f.str)
        f.next()
        out.append((master, _stoi(f.str)))
    return out


def conditions_arrays(conds):
    """(node, dof, value) arrays of a ((node, dof), value) list, for FemMesh.set_dirichlet and
    FemMesh.set_loads."""
    n = np.array([c[0][0] for c in conds], np.int32)
    d = np.array([c[0][1] for c in conds], np.int32)
    v = np.array([c[1] for c in conds], float)
    return n, d, v

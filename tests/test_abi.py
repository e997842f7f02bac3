"""C-ABI library: loads on a host without a GPU, exports every declared entry point, and its
host-side logic (ghost bookkeeping, argument checks) matches the reference (through the oracle).
No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle_dsl as O
import spatialops_gb300 as N

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for h in sorted(os.listdir(os.path.join(REPO, "include"))):
        if not h.endswith(".h"):
            continue
        txt = open(os.path.join(REPO, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"\b(nebo_[a-z0-9_]+)\s*\(", txt)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = N.lib()
    names = declared_symbols()
    assert len(names) >= 15
    for name in names:
        assert hasattr(L, name), name


def test_python_signatures_cover_header():
    assert set(declared_symbols()) == {s[0] for s in N.SIGNATURES}


def test_status_strings():
    L = N.lib()
    assert L.nebo_status_string(0) == b"ok"
    assert b"ghost" in L.nebo_status_string(2)


def test_null_descriptor_is_rejected_without_gpu():
    L = N.lib()
    rc = L.nebo_heat_step(None, None, None, 0.1, None, None)
    assert rc == 1
    assert b"null field descriptor" in L.nebo_last_error()


def _header_enum(name):
    txt = open(os.path.join(REPO, "include", "nebo_gb300.h")).read()
    return int(re.search(r"\b%s\s*=\s*(0x[0-9a-fA-F]+|-?\d+)" % name, txt).group(1), 0)


def test_heat_modes_match_header():
    assert N.HEAT_MODES == {"exact": _header_enum("NEBO_HEAT_EXACT"), "fixed": _header_enum("NEBO_HEAT_FIXED_POINT"),
                            "fixed_state": _header_enum("NEBO_HEAT_FIXED_STATE")}
    assert N.HEAT_GRAPH == _header_enum("NEBO_HEAT_GRAPH")
    assert not any(v & N.HEAT_GRAPH for v in N.HEAT_MODES.values())


@pytest.mark.parametrize("mode", [7, 7 | 0x100])
def test_heat_run_ex_rejects_an_unknown_mode_without_gpu(mode):
    L = N.lib()
    rc = L.nebo_heat_run_ex(None, None, None, 1, 0.1, None, mode, None)
    assert rc == 1
    assert b"mode 7" in L.nebo_last_error()


def _rand_expr(rng, fields, depth, db):
    """Random Nebo expression over SVol fields (pointwise ops, cond, same-type stencils)."""
    if depth == 0 or rng.random() < 0.2:
        return fields[rng.integers(len(fields))] if rng.random() < 0.8 else O.Scalar(1.5)
    k = rng.integers(5)
    a = _rand_expr(rng, fields, depth - 1, db)
    if k == 0:
        return a + _rand_expr(rng, fields, depth - 1, db)
    if k == 1:
        return O.sin(a)
    if k == 2:
        return O.cond(a > 0.0, a, _rand_expr(rng, fields, depth - 1, db))
    if k == 3:
        return db.fd("grad", int(rng.integers(3)))(a)
    return db.filter()(a)


@pytest.mark.parametrize("ghost,bc", [(1, (0, 0, 0)), (2, (0, 0, 0)), (1, (1, 0, 1)), (3, (1, 1, 1))])
def test_write_limits_match_reference_rule(ghost, bc):
    n = (9, 8, 7)
    rng = np.random.default_rng(ghost * 10 + sum(bc))
    g = O.glob_dims("SVol", n, ghost, bc)
    fields = [O.Field("SVol", np.zeros((g[2], g[1], g[0])), ghost, bc) for _ in range(3)]
    db = O.OpDB(n, n)
    lhs_o = O.Field("SVol", np.zeros((g[2], g[1], g[0])), ghost, bc)
    lhs_n = N.Field.__new__(N.Field)
    lhs_n.loc, lhs_n.n, lhs_n.ghost, lhs_n.bc, lhs_n.dtype, lhs_n.glob = "SVol", n, ghost, bc, N.F64, g
    for trial in range(60):
        e = _rand_expr(rng, fields, 4, db)
        use_ghost = bool(rng.integers(2))
        m, p = O.ghosts(e, True)
        d = N.NeboField()
        d.data = 1
        d.glob[:] = g
        d.extent[:] = g
        d.ghost_minus[:] = (ghost,) * 3
        d.ghost_plus[:] = (ghost,) * 3
        d.has_bc[:] = bc
        d.bc_extra[:] = (0, 0, 0)
        try:
            lo, _ = O.write_limits(lhs_o, e, use_ghost)
            ref_err = None
        except O.NeboError as ex:
            ref_err = str(ex)
        try:
            got = N.write_limits(d, m, p, use_ghost)
            got_err = None
        except RuntimeError as ex:
            got_err = str(ex)
        assert (ref_err is None) == (got_err is None)
        if ref_err is None:
            assert got == lo

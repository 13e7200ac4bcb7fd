"""Input-file handling of the drivers (drivers.load_inputs, the restart-parameter round trip)
on the CPU: the reference's load_inputs semantics (sscanf "key = %lf" / "%i" per line,
comments, unread lines reported, command-line overrides last) and its refusals."""
import math

import pytest

import drivers as D
import h5io

INPUT = """# test input in the reference's format
#### Problem Specification ####
xl = 0.0           # spatial domain
xr=2.5
nx = 64            # grid
ny = 010           # %i reads a leading 0 as octal
nz = 0x10
xlbc = 3
xrbc = 3
tf = 0.2
gamma = 1.4
nout = 4
showstats = 1
rtol = 1e-5
atol = 1e-12
mxsteps = 10000
order = 3.9        # %i stops at the point
htrans = .5e-3
bogus = 7
  nx = 99          # not at the start of the line: sscanf does not read it
"""


def _write(tmp_path, text=INPUT):
    p = tmp_path / "input.txt"
    p.write_text(text)
    return str(p)


def test_defaults():
    inp = D.load_inputs()
    assert inp.u == D.UDATA_DEFAULTS and inp.o == D.OPTS_DEFAULTS and inp.restart == -1
    assert inp.o["rtol"] == 1e-8 and inp.o["mxsteps"] == 5000 and inp.u["nout"] == 10


def test_file_semantics(tmp_path):
    inp = D.load_inputs(_write(tmp_path))
    u, o = inp.u, inp.o
    assert u["xr"] == 2.5 and u["nx"] == 64 and u["ny"] == 8 and u["nz"] == 16
    assert u["xlbc"] == 3 and u["tf"] == 0.2 and u["nout"] == 4 and u["showstats"] == 1
    assert o["rtol"] == 1e-5 and o["mxsteps"] == 10000 and o["order"] == 3
    assert o["htrans"] == 5e-4
    assert isinstance(u["nx"], int) and isinstance(o["rtol"], float)
    # the unread line is reported, the indented one is not read and contains '='
    assert any(w.startswith("bogus") for w in inp.warnings)
    assert inp.shape == (16, 8, 64) and inp.bc == (3, 3, 0, 0, 0, 0)
    assert inp.domain == (0.0, 2.5, 0.0, 1.0, 0.0, 1.0)


def test_overrides_take_precedence(tmp_path):
    inp = D.load_inputs(_write(tmp_path), nx=128, rtol=1e-7, restart=3)
    assert inp.u["nx"] == 128 and inp.o["rtol"] == 1e-7 and inp.restart == 3
    with pytest.raises(ValueError):
        D.load_inputs(_write(tmp_path), no_such_option=1)


def test_refusals(tmp_path):
    with pytest.raises(ValueError, match="hmax"):
        D.load_inputs(fixedstep=1)
    with pytest.raises(ValueError):
        D.load_inputs(nout=0)
    with pytest.raises(ValueError):
        D.load_inputs(TimeUnits=0.0)
    # MRI coupling numbers this package does not have, and inner fixed steps
    with pytest.raises(ValueError, match="mtable"):
        D.run_multirate(D.load_inputs(mtable=202, itable=112), None, None)
    with pytest.raises(ValueError, match="fixedstep"):
        D.run_multirate(D.load_inputs(fixedstep=1, hmax=1e-3, itable=112), None, None)


def test_restart_parameters_round_trip(tmp_path):
    inp = D.load_inputs(_write(tmp_path))
    params = inp.params()
    assert {k for k, _ in h5io.PARAMETERS} <= set(params)
    h5io.write_parameters(str(tmp_path), params, tcur=0.1, hcur=1.2345678901234567e-3, iout=2)
    back = D.load_inputs(str(tmp_path / "restart_parameters.txt"))
    assert back.restart == 2 and back.u["t0"] == 0.1 and back.o["h0"] == 1.2345678901234567e-3
    assert back.u["nout"] == inp.u["nout"] - 2
    for k in ("nx", "ny", "nz", "xr", "tf", "gamma", "xlbc"):
        assert back.u[k] == inp.u[k], k
    for k in ("rtol", "atol", "mxsteps", "order", "htrans"):
        assert back.o[k] == inp.o[k], k
    assert not back.warnings


def test_scan_matches_sscanf_rules():
    assert D._scan(" 12abc", True) == 12 and D._scan("-0x1f", True) == -31
    assert D._scan("017", True) == 15 and D._scan("0", True) == 0 and D._scan("x", True) is None
    assert D._scan("1e-3 # c", False) == 1e-3 and D._scan("-.5", False) == -0.5
    assert D._scan("5e", False) == 5.0 and math.isinf(D._scan("inf", False))
    assert D._match("xlbc = 1", "xl") is None and D._match("xl= 3", "xl").strip() == "3"


def test_method_selection_follows_the_inputs():
    """order overrides etable for the hydro driver (ARKODE's default table of each order);
    the chemistry drivers take ARKStepSetTableNum(itable, etable); unknown numbers refused."""
    import integrate as I
    assert D.erk_table(D.load_inputs(order=4).o) == 3          # Zonneveld 5-3-4
    assert D.erk_table(D.load_inputs(order=5).o) == 6          # Cash-Karp 6-4-5
    assert D.erk_table(D.load_inputs(order=0, etable=13).o) == 13
    assert D.erk_table(D.load_inputs(order=0, etable=8).o) == 8
    assert D.erk_table(D.load_inputs(order=0).o) == 3
    for bad in (dict(order=7), dict(order=0, etable=5)):
        with pytest.raises(Exception):
            D.erk_table(D.load_inputs(**bad).o)
    # the primordial inputs' IMEX pair and static-chemistry DIRK-only setting
    t = I.ark_table(13, 112)
    assert t["name"] == "ARK437L2SA_ERK_7_3_4+ARK437L2SA_DIRK_7_3_4"
    assert not I.ark_table(-1, 112)["explicit"]
    with pytest.raises(ValueError):
        D.run_imex(D.load_inputs(etable=-1, itable=-1), None, None)
    with pytest.raises(ValueError, match="itable"):
        D.run_multirate(D.load_inputs(itable=-1), None, None)
    # the controller options reach the integrators
    kw = D._adapt(D.load_inputs(adapt_method=2, safety=0.99, bias=2.0, growth=2.0).o)
    assert kw == {"adapt_method": 2, "pq": 0, "safety": 0.99, "bias": 2.0, "growth": 2.0}

"""Input-file compatibility (apps/hydro/inputs.h:100-135) and the command-line
driver's options (apps/common/arguments.h:25-70): the Lua "hydro" table, its
eos sub-table, the ics function and the box mesh table, read by the library's
Lua-subset interpreter."""
import os
import subprocess

import numpy as np
import pytest

import flecsale_gb300.hydro as H
from tests import _util as U

INPUTS = os.path.join(U.GOLDEN, "inputs")


def test_shock_box_2d_input():
    inp = H.Input(os.path.join(INPUTS, "shock_box_2d.lua"))
    p, max_steps, output_freq = inp.params(2)
    assert (p.cfl, p.final_time, p.gamma, p.cv) == (0.5, 0.2, 1.4, 1.0)
    assert (max_steps, output_freq) == (20, 1000000)   # "1e6" is a numeric string
    assert inp.string("hydro.prefix") == "shock_box_2d"
    assert inp.number("hydro.eos.gas_constant") == 1.4
    mesh = H.HostMesh.box(2, (8, 6), [-0.5, -0.5], [0.5, 0.5])
    s = inp.initial_state(mesh, p)
    ref = H.initial_state("shock_box", mesh, p)   # apps/hydro/2d/inputs.cc:45-60
    assert np.array_equal(s, ref)


def test_shock_box_3d_input_with_mesh_table():
    inp = H.Input(os.path.join(INPUTS, "shock_box_3d_box.lua"))
    p, max_steps, _ = inp.params(3)
    assert abs(p.cfl - 1.0 / 3.0) < 1e-16 and max_steps == 12
    mesh = inp.mesh()
    assert (mesh.dim, mesh.num_cells) == (3, 1000)
    cc = mesh.arrays()["cell_centroid"]
    assert np.isclose(cc.min(), -0.45) and np.isclose(cc.max(), 0.45)
    s = inp.initial_state(mesh, p)
    assert np.array_equal(s, H.initial_state("shock_box", mesh, p))


@pytest.mark.parametrize("name", ["2d/shock_box_2d.lua", "3d/shock_box_3d.lua"])
def test_reference_input_files(name):
    path = os.path.join(U.REFERENCE, "apps/hydro", name)
    if not os.path.exists(path):
        pytest.skip("reference checkout not present")
    inp = H.Input(path)
    dim = 2 if name.startswith("2d") else 3
    p, max_steps, output_freq = inp.params(dim)
    assert max_steps in (12, 20) and output_freq == 1000000 and p.gamma == 1.4
    mesh = inp.mesh() if dim == 3 else H.HostMesh.box(2, (4, 4), [-0.5, -0.5], [0.5, 0.5])
    assert np.array_equal(inp.initial_state(mesh, p), H.initial_state("shock_box", mesh, p))


LANG = r"""
-- a line comment
--[[ a block
     comment ]]
local helper = 3
hydro = {
  prec = {2^3^2, -2^2, 1 + 2 * 3, (1 + 2) * 3, 7 % 3, -7 % 3, 2 * -3, 10 / 4},
  logic = {1 < 2 and "yes" or "no", nil or 5, false and 1, not nil, 1 == 1.0, "a" ~= "b"},
  str = "tab\there" .. [[ long]] .. 'q' .. 1,
  nested = {a = {b = {c = 42}}, [3] = "third", [1] = "first", "x"},
  f = function (n)
    local acc = 0
    for i = 1, n do acc = acc + i end
    local k = 0
    while k < 10 do k = k + 3 end
    if n > 100 then return -1 elseif n > 5 then return acc, k else return 0 end
  end,
  g = function () local function sq(x) return x * x end return sq(helper), math.sqrt(16), math.max(1, 9, 4), math.pi end,
  closure = (function () local c = 10 return function (d) c = c + d return c end end)(),
  semi = 1; other = 2,
}
"""


def test_interpreter_semantics():
    inp = H.Input(text=LANG)
    prec = [inp.number(f"hydro.prec[{i}]") for i in range(1, 9)]
    assert prec == [512, -4, 7, 9, 1, 2, -6, 2.5]
    assert inp.string("hydro.logic[1]") == "yes" and inp.number("hydro.logic[2]") == 5
    assert inp.string("hydro.str") == "tab\there longq1"
    assert inp.number("hydro.nested.a.b.c") == 42
    assert inp.string("hydro.nested[1]") == "x"          # positional entries win over [1]
    assert inp.string("hydro.nested[3]") == "third"
    assert inp.number("hydro.semi") == 1 and inp.number("hydro.other") == 2


def test_interpreter_errors():
    with pytest.raises(H.FvhError, match=r"input:3: "):
        H.Input(text="hydro = {\n a = 1,\n b = = 2 }")
    with pytest.raises(H.FvhError, match="no table 'hydro'"):
        H.Input(text="x = 1")
    with pytest.raises(H.FvhError, match="attempt to call"):
        H.Input(text="hydro = {}\nlocal y = undefined_fn(1)")
    inp = H.Input(text="hydro = { eos = { type = 'stiffened_gas' } }")
    with pytest.raises(H.FvhError):
        inp.params(2)
    with pytest.raises(H.FvhError):
        H.Input(path="/nonexistent/input.lua")


def test_ics_function_errors():
    mesh = H.HostMesh.box(2, (2, 2), [0, 0], [1, 1])
    p = H.make_params(2)
    bad = H.Input(text="hydro = { ics = function (x, y, t) return 1.0 end }")
    with pytest.raises(H.FvhError):
        bad.initial_state(mesh, p)


def test_driver_options():
    drv = H.driver_path()
    r = subprocess.run([drv, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "--input_file" in r.stdout and "--mesh" in r.stdout
    r = subprocess.run([drv, "--flux", "roe"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    r = subprocess.run([drv, "-f", "/nonexistent.lua"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "cannot open" in r.stderr


_HOSTILE = r'''
import sys
import flecsale_gb300.hydro as H

def load(text):
    try:
        H.Input(text=text + "\nhydro = {}").close()
        return "ok"
    except H.FvhError as e:
        return "error: " + str(e)[:60]

n = 200000
cases = {
    "parens": "x = " + "(" * n + "1" + ")" * n,
    "unary": "x = " + "- " * n + "1",
    "sum": "x = 1" + " + 1" * n,
    "power": "x = 2" + " ^ 1" * n,
    "concat": "x = 'a'" + " .. 'a'" * n,
    "suffix": "t = {} x = t" + ".a" * n,
    "calls": "f = function() return f end x = f" + "()" * n,
    "tables": "x = " + "{" * n + "}" * n,
    "blocks": "do " * n + "end " * n,
    "functions": "x = " + "function() return " * 5000 + "1" + " end" * 5000,
    "recursion": "function f(k) return f(k + 1) end f(1)",
    "deep_body": "function f(k) if k > 0 then return " + "(" * 400 + "f(k - 1)" + ")" * 400
                 + " end return 0 end x = f(150)",
}
# data chains built at run time are freed without recursing per link
runtime = {
    "table_chain": "local t = {} for i = 1, 300000 do t = {t} end x = t",
    "closure_chain": "local f = nil for i = 1, 300000 do local g = f f = function() return g end end x = f",
    "many_locals": "local a = 1\n" * 100000 + "x = a",
}
for name, text in list(cases.items()) + list(runtime.items()):
    print(name, load(text), flush=True)
print("survived")
'''


def test_hostile_inputs_are_refused_not_crashed():
    """Nesting far beyond any input file (parentheses, operator and suffix
    chains, tables, blocks, recursion) is refused with an error, and long
    chains of tables or closures built at run time are freed without
    overflowing the native stack (checked in a child process)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([os.sys.executable, "-c", _HOSTILE], capture_output=True, text=True,
                       timeout=600, cwd=root, env=dict(os.environ, PYTHONPATH=root))
    assert r.returncode == 0 and "survived" in r.stdout, (r.returncode, r.stdout[-3000:],
                                                          r.stderr[-3000:])
    lines = dict(l.split(" ", 1) for l in r.stdout.splitlines() if " " in l)
    for name in ("parens", "unary", "sum", "power", "concat", "suffix", "calls", "tables",
                 "blocks", "functions"):
        assert "too many syntax levels" in lines[name], (name, lines[name])
    for name in ("recursion", "deep_body"):
        assert "stack overflow" in lines[name], (name, lines[name])
    for name in ("table_chain", "closure_chain", "many_locals"):
        assert lines[name] == "ok", (name, lines[name])


def test_input_mesh_and_initial_state_values_are_checked():
    """Box dimensions must be whole cell counts that int32 holds, extents
    finite; the ics function must return positive, finite density and
    pressure and finite velocity (the reference asserts rho > 0 and p > 0,
    euler_eqns.h:342-343).  Each violation is an error status."""
    base = "hydro = {{ mesh = {{ type = 'box', dimensions = {{{dims}}}, xmin = {{0, 0}}, " \
           "xmax = {{{xmax}, 1}} }}, ics = function(x, y, t) return {ret} end }}"
    good = dict(dims="4, 3", xmax="1", ret="1.0, {0.5, 0}, 2.0")
    inp = H.Input(text=base.format(**good))
    mesh = inp.mesh()
    p, _, _ = inp.params(2)
    s = inp.initial_state(mesh, p)
    assert mesh.num_cells == 12 and np.all(s[0] == 1.0) and np.all(s[1] == 0.5)
    for dims in ("4.5, 3", "0, 3", "-2, 3", "0/0, 3", "1e12, 3"):
        with pytest.raises(H.FvhError):
            H.Input(text=base.format(**dict(good, dims=dims))).mesh()
    for xmax in ("1/0", "0/0", "-1"):
        with pytest.raises(H.FvhError):
            H.Input(text=base.format(**dict(good, xmax=xmax))).mesh()
    for ret in ("0.0, {0, 0}, 1.0", "1.0, {0, 0}, -1.0", "0/0, {0, 0}, 1.0",
                "1.0, {1/0, 0}, 1.0", "1.0, {0, 0}, 1/0"):
        bad = H.Input(text=base.format(**dict(good, ret=ret)))
        with pytest.raises(H.FvhError):
            bad.initial_state(mesh, p)


def test_mutated_input_files_are_loaded_or_refused():
    """Random byte mutations of the shipped input files either load or are
    refused with an error status, never crash (in a child process); an error
    message quoting a byte that is not UTF-8 still reaches Python as FvhError."""
    with pytest.raises(H.FvhError):
        H.Input(text="x = \x80\nhydro = {}")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([os.sys.executable, os.path.join(root, "tests", "_lua_fuzz.py"), "5", "1500"],
                       capture_output=True, text=True, timeout=600, cwd=root,
                       env=dict(os.environ, PYTHONPATH=root))
    assert r.returncode == 0, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])
    assert "refused" in r.stdout


def test_input_parameter_values_are_checked():
    """Out-of-range values in the hydro table are refused (and p is left as
    it was); numeric strings such as output_freq = "1e6" still read."""
    ok = H.Input(text="hydro = { CFL = 0.3, final_time = 0.1, max_steps = 7, output_freq = '1e6',"
                      " eos = { type = 'ideal_gas', gas_constant = 1.6, specific_heat = 2 } }")
    p, ms, of = ok.params(2)
    assert (p.cfl, p.final_time, p.gamma, p.cv, ms, of) == (0.3, 0.1, 1.6, 2.0, 7, 1000000)
    bad = ["CFL = -1", "CFL = 0/0", "CFL = 1/0", "final_time = 0/0", "max_steps = -1",
           "max_steps = 1.5", "max_steps = 0/0", "max_steps = 1e300", "output_freq = -3",
           "eos = { type = 'ideal_gas', gas_constant = 1 }",
           "eos = { type = 'ideal_gas', specific_heat = 0 }"]
    for entry in bad:
        inp = H.Input(text=f"hydro = {{ {entry} }}")
        with pytest.raises(H.FvhError) as e:
            inp.params(2)
        assert e.value.code == H.ERR_INVALID_ARGUMENT, entry
    with pytest.raises(H.FvhError) as e:
        H.Input(text="hydro = { eos = { type = 'stiffened_gas' } }").params(2)
    assert e.value.code == H.ERR_UNSUPPORTED

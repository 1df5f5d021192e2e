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

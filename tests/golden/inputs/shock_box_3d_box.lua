-- 3D shock box with the mesh given as a box table (the form of
-- apps/hydro/3d's input), a 10^3 hexahedral box on [-0.5, 0.5]^3.
hydro = {
  prefix = "shock_box_3d",
  postfix = "dat",
  output_freq = 1e6,
  final_time = 0.2,
  max_steps = 12,
  CFL = 1./3.,
  mesh = {
    type = "box",
    dimensions = {10, 10, 10},
    xmin = {-0.5, -0.5, -0.5},
    xmax = { 0.5,  0.5,  0.5}
  },
  eos = { type = "ideal_gas", gas_constant = 1.4, specific_heat = 1.0 },
  ics = function (x, y, z, t)
    local inside = x < 0 and y < 0 and z < 0
    if inside then
      return 0.125, {0, 0, 0}, 0.1
    else
      return 1.0, {0, 0, 0}, 1.0
    end
  end
}

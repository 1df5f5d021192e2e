-- 2D shock box of apps/hydro/2d as an input file: the parameters of
-- apps/hydro/2d/inputs.cc, in the hydro-table form inputs.h reads.
hydro = {
  prefix = "shock_box_2d",
  postfix = "dat",
  output_freq = "1e6",          -- a numeric string, as in the reference's file
  final_time = 0.2,
  max_steps = 20,
  CFL = 1./2.,
  eos = {
    type = "ideal_gas",
    gas_constant = 1.4,
    specific_heat = 1.0,
  },
  -- density, velocity, pressure at a cell centroid
  ics = function (x, y, t)
    if x < 0 and y < 0 then
      return 0.125, {0, 0}, 0.1
    end
    return 1.0, {0, 0}, 1.0
  end,
}

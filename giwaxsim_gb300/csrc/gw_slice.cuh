// Per-column arithmetic shared by the voxel stage and the standalone
// rectangular_collapse_lengths entry point.
#pragma once

#include "gw_common.cuh"

// rectangular_collapse_lengths (voxelgrids.py:238-309) at column x_val.
__host__ __device__ inline double collapse_length(const gw_phi &ph, double hor, double ver,
                                  double base, double x) {
  if (ph.cl_swap) { double t = hor; hor = ver; ver = t; }
  if (ph.cl_case == 0) return x < hor ? ver : 0.0;
  if (ph.cl_case == 1) return x < ver ? hor : 0.0;
  const double vc = GW_DMUL(ver, ph.cos_t);
  double stop1 = vc, stop2 = GW_DMUL(hor, ph.cos_p), mid;
  if (stop1 < stop2) {
    mid = GW_DDIV(ver, ph.sin_t);
  } else {
    double t = stop1; stop1 = stop2; stop2 = t;
    mid = GW_DDIV(hor, ph.sin_p);
  }
  if (x == 0.0) return 0.0;
  if (x < stop1) {
    const double tot = GW_DADD(base, GW_DMUL(x, ph.tan_p));
    const double miss = GW_DMUL(GW_DSUB(vc, x), ph.tan_t);
    return GW_DSUB(tot, miss);
  }
  if (x <= stop2) return mid;
  if (x < GW_DADD(stop1, stop2)) {
    const double rem = GW_DSUB(hor, GW_DDIV(GW_DSUB(x, vc), ph.cos_p));
    return GW_DDIV(rem, ph.cos_t);
  }
  return 0.0;
}


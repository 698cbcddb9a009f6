// bc.cuh -- boundary nodes of the structured RVE grid and the affine boundary fields of unit strains.
#pragma once

#include "device.cuh"

namespace mgb {

// Grid coordinates of node n; true when it lies on the boundary (its rows are Dirichlet rows).
__device__ __forceinline__ bool bnd(const MeshDev &m, int n, int &i, int &j, int &k) {
  i = n % m.nx;
  j = (n / m.nx) % m.ny;
  k = n / m.nxny;
  return i == 0 || j == 0 || k == 0 || i == m.nx - 1 || j == m.ny - 1 || k == m.nz - 1;
}

// Coordinates a boundary node takes in the affine boundary condition (same face priority as k_set_bc).
__device__ __forceinline__ void bc_coords(const MeshDev &m, int i, int j, int k, double c[3]) {
  if (i == m.nx - 1) {
    c[0] = m.lx; c[1] = j * m.dy; c[2] = k * m.dz;
  } else if (i == 0) {
    c[0] = 0; c[1] = j * m.dy; c[2] = k * m.dz;
  } else if (j == m.ny - 1) {
    c[0] = i * m.dx; c[1] = m.ly; c[2] = k * m.dz;
  } else if (j == 0) {
    c[0] = i * m.dx; c[1] = 0; c[2] = k * m.dz;
  } else if (k == m.nz - 1) {
    c[0] = i * m.dx; c[1] = j * m.dy; c[2] = m.lz;
  } else {
    c[0] = i * m.dx; c[1] = j * m.dy; c[2] = 0;
  }
}

// Boundary displacement of the unit Voigt strain e_r (engineering shear: e_3 gives eps_xy = 1/2).
__device__ __forceinline__ void lift(const double c[3], int r, double w[3]) {
  w[0] = w[1] = w[2] = 0.0;
  switch (r) {
    case 0: w[0] = c[0]; break;
    case 1: w[1] = c[1]; break;
    case 2: w[2] = c[2]; break;
    case 3: w[0] = 0.5 * c[1]; w[1] = 0.5 * c[0]; break;
    case 4: w[0] = 0.5 * c[2]; w[2] = 0.5 * c[0]; break;
    default: w[1] = 0.5 * c[2]; w[2] = 0.5 * c[1]; break;
  }
}

}  // namespace mgb

/* material.c -- material_set / material_print of the micropp3 C ABI (include/material_base.h).
 * The derived constants use the expressions of the reference's material.c:26-38. */
#include <stdio.h>

#include "material_base.h"

void material_set(struct material_base *self, const int type, const double E, const double nu, const double Ka,
                  const double Sy, const double Xt) {
  self->E = E;
  self->nu = nu;
  self->Ka = Ka;
  self->Sy = Sy;
  self->Xt = Xt;
  self->type = type;
  self->k = E / (3. * (1. - 2. * nu));
  self->mu = E / (2. * (1. + nu));
  self->lambda = nu * E / ((1. + nu) * (1. - 2. * nu));
}

void material_print(const struct material_base *self) {
  printf("E = %e\nnu = %e\nKa = %e\nSy = %e\nXt = %e\nk = %e\nmu = %e\nlambda = %e\ntype = %1d\n", self->E, self->nu,
         self->Ka, self->Sy, self->Xt, self->k, self->mu, self->lambda, self->type);
}

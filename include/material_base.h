/*
 * material_base.h -- material record of the micropp3 C/Fortran ABI.
 *
 * Drop-in for the reference's include/material_base.h:27-55: the same enum, struct layout (which the
 * Fortran binding mirrors, material.f95:30-35) and the two C entry points.
 */
#ifndef MICROPP_GB300_MATERIAL_BASE_H
#define MICROPP_GB300_MATERIAL_BASE_H

enum { MATERIAL_ELASTIC = 0, MATERIAL_PLASTIC, MATERIAL_DAMAGE };

#ifdef __cplusplus
extern "C" {
#endif

struct material_base {
  double E, nu, Ka, Sy;
  double k, mu, lambda;
  double Xt;
  int type;
};

/* Replaces material_set (material_base.h:47-48, material.c:26-38): stores the parameters and derives the
 * bulk modulus k and the Lame constants mu, lambda. */
void material_set(struct material_base *self, const int type, const double E, const double nu, const double Ka,
                  const double Sy, const double Xt);

/* Replaces material_print (material_base.h:50, material.c:40-45). */
void material_print(const struct material_base *self);

#ifdef __cplusplus
}
#endif
#endif

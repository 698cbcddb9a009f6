/*
 * micropp_c.h -- the micropp3 C ABI, served by the GB300 library (libmicropp_gb300.so).
 *
 * Every declaration replaces the entry point of the same name in the reference's include/micropp_c.h
 * (cited per entry); argument meaning and (void) error behaviour are the same, so a macro-scale code
 * (C, C++, or Fortran through iso_c_binding as in micropp.f95:37-180) relinks unchanged.  GPU failures that
 * the reference cannot have are reported on stderr and through micropp3_last_error() (micropp_gb300.h).
 */
#ifndef MICROPP_GB300_MICROPP_C_H
#define MICROPP_GB300_MICROPP_C_H

#include <stdbool.h>

#include "material_base.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Opaque handle (micropp_c.h:33-35). */
struct micropp3 {
  void *ptr;
};

/* micropp_c.h:37-39 / micropp_c.cpp:33-58.  As in the reference wrapper, sub-iterations are switched on,
 * A0 reuse and the profiling log are off, and every other parameter keeps its micropp_params_t default;
 * `micro_params` holds 4 geometry parameters, `materials` 3 records and `coupling` ngp entries. */
void micropp3_new(struct micropp3 *self, int ngp, const int size[3], const int micro_type, const double *micro_params,
                  const struct material_base *materials, const int *coupling, const int nsubiterations,
                  const int mpi_rank);

/* micropp_c.h:41 */
void micropp3_free(struct micropp3 *self);

/* micropp_c.h:43: the 6 Voigt components (xx, yy, zz, xy, xz, yz; engineering shear) of macro point gp. */
void micropp3_set_strain(struct micropp3 *self, const int gp_id, const double *strain);

/* micropp_c.h:45: the 6 volume-averaged stress components of the last homogenize(). */
void micropp3_get_stress(const struct micropp3 *self, const int gp_id, double *stress);

/* micropp_c.h:47: the 6x6 tangent, row-major, column i = d(stress)/d(strain_i). */
void micropp3_get_ctan(const struct micropp3 *self, const int gp_id, double *ctan);

/* micropp_c.h:49: homogenize every macro point of the handle (all RVEs batched on the GPU). */
void micropp3_homogenize(struct micropp3 *self);

/* micropp_c.h:51: stress = ctan * strain for every point, without an FE solve. */
void micropp3_homogenize_linear(struct micropp3 *self);

/* micropp_c.h:53: accept the last step (swap history and displacement buffers). */
void micropp3_update_vars(struct micropp3 *self);

/* micropp_c.h:55-65 */
bool micropp3_is_non_linear(const struct micropp3 *self, const int gp_id);
int micropp3_get_cost(const struct micropp3 *self, int gp_id);
bool micropp3_has_converged(const struct micropp3 *self, int gp_id);
bool micropp3_has_subiterated(const struct micropp3 *self, int gp_id);

/* micropp_c.h:63: VTU output of one RVE (displacement, element strain/stress, phase). */
void micropp3_output(struct micropp3 *self, const int gp_id, const char *filename);

/* micropp_c.cpp:113-116 (declared only by the Fortran binding, micropp.f95:148-156). */
void micropp3_output2(struct micropp3 *self, const int gp_id, const int elem_global, const int time_step);

/* micropp_c.h:65 */
void micropp3_print_info(struct micropp3 *self);

/* micropp_c.h:67 */
int micropp3_get_non_linear_gps(const struct micropp3 *self);

/* micropp_c.h:69-70: micropp-restart-<mpi_rank>-<restart_id>.bin in the reference's binary format. */
void micropp3_write_restart(const struct micropp3 *self, const int restart_id);
void micropp3_read_restart(const struct micropp3 *self, const int restart_id);

#ifdef __cplusplus
}
#endif
#endif

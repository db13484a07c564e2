/* athena_gb300 diagnostics: timing and self-check entry points of libathgpu.so.
 *
 * None of these replaces an interface of the reference: they time the library's own
 * kernels and check its device arithmetic against the hardware and the solvers against
 * stated references.  The stage update does not need them; the product interface is
 * athena_gb300.h. */
#ifndef ATHENA_GB300_DIAG_H_
#define ATHENA_GB300_DIAG_H_

#include "athena_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Run one cycle without the CUDA graph, timing every kernel launch with CUDA events on
 * the context's stream; ms[i] (i < cap) receives the duration of launch i, *count the
 * number of launches, athgpu_profile_label(ctx, i) its kernel name.  The state advances
 * by one cycle.  Synchronous. */
athgpu_status athgpu_profile_cycle(athgpu_ctx *ctx, int cap, float *ms, int *count);
const char *athgpu_profile_label(athgpu_ctx *ctx, int idx);

/* Number of kernels the library launched since the last reset. */
athgpu_status athgpu_launch_count(athgpu_ctx *ctx, long long *count, int reset);

/* Host wall milliseconds of the phases of the last athgpu_regrid: ms[8] = new registers
 * (queued), restriction on the old mesh, box copies (queued), prolongation (queued),
 * multi-level plan (built on the host while the queued work runs, then the wait for it),
 * release of the old registers, Initialize(2), (unused). */
athgpu_status athgpu_regrid_profile(double* ms);

/* Self-check of the FP64 <-> FP32 arithmetic the FP32 kernels do on the integer pipe
 * (GB300's FP64 pipe, which also runs the conversion instructions, is narrow): for device
 * arrays d[n], f[n], mismatches[0] (device) receives the number of d[q] whose integer-pipe
 * rounding to float differs bitwise from the hardware's, mismatches[1] the same for the
 * widening of f[q], mismatches[2] the same for the FP64 difference of the pair
 * (f[q], f[q ^ 1]) that the FP32 CT update forms.  No counterpart in the reference. */
athgpu_status athgpu_selftest_conversions(long long n, const double *d, const float *f,
                                          unsigned long long *mismatches, void *stream);

/* Self-check of the Riemann solvers on arbitrary face states: for device arrays wl[n][7],
 * wr[n][7] (primitive states in the solvers' local order: density, normal and two
 * transverse velocities (relativistic: spatial 4-velocity), gas pressure, two transverse
 * fields), bx[n] (normal field), flux[n][7] (device) receives each face's flux in the same
 * order (mass, three momenta, energy, then the two transverse-field fluxes, before the
 * EMF sign flip of the caller).  dv[n][2] (device, may be NULL for zeros): each face's
 * velocity differences (dvn, dvt) that ATHGPU_LHLLD reads (the other solvers ignore them).
 * rsolver as in athgpu_mesh_desc; FP64.  Replaces no
 * reference interface: the solvers' own entry points are the per-pencil RiemannSolver
 * functions (hydro/rsolvers/mhd/*.cpp), which this applies one face at a time.
 * Asynchronous on `stream`. */
athgpu_status athgpu_selftest_riemann(int rsolver, int relativistic, double gamma,
                                      long long n, const double *wl, const double *wr,
                                      const double *bx, const double *dv, double *flux,
                                      void *stream);

/* The same in FP32 (float arrays, same layout), with the solvers the FP32 sweeps run
 * (HLLD and HLLE: the packed left/right forms).  Replaces no reference interface. */
athgpu_status athgpu_selftest_riemann_fp32(int rsolver, int relativistic, double gamma,
                                           long long n, const float *wl, const float *wr,
                                           const float *bx, const float *dv, float *flux,
                                           void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ATHENA_GB300_DIAG_H_ */

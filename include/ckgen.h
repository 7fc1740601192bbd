/*
 * ckgen.h — synthetic event generator for the CudaKalman workloads.
 *
 * Plays the role the reference gives to Fatras + digitisation for its
 * truth-tracking examples (Fatras/, Examples/Scripts/Python/
 * truth_tracking_kalman.py): it builds the detector (surface table), the
 * magnetic field and, per track, the truth trajectory, the surface sequence
 * the truth crosses, smeared 2D measurements (with holes and outliers on
 * request) and smeared start parameters. Output arrays have the layout of
 * ck_batch_in (include/cudakalman.h).
 *
 * Deterministic: every track draws from its own counter-based stream seeded
 * by (seed, track id), so results do not depend on thread count or batch
 * splitting.
 */
#ifndef CKGEN_H
#define CKGEN_H

#include <stdint.h>

#include "cudakalman.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Workload presets (the five benchmark configurations of this fitter). */
enum {
  CKG_TELESCOPE = 1,   /* 10 planes x = 30..300 mm, no material, 2 T, muons  */
  CKG_BARREL = 2,      /* 10 Si cylinders r = 32..1020 mm, 2 T, pions        */
  CKG_BARREL_MIXED = 3,/* geometry and tracks of CKG_BARREL                  */
  CKG_UNEVEN = 4,      /* 20 Si cylinders, grid field, 4-20 hits, holes,
                          outliers                                         */
  CKG_SERVING = 5,     /* tracks of CKG_UNEVEN                               */
  CKG_STRIPS = 6       /* geometry, field and tracks of CKG_BARREL; the outer
                          six layers are read out by strips: 1D measurements
                          of loc0 (100 um) and loc1 (150 um) on alternate
                          layers, as the reference's KF test detector
                          (FitterTestsCommon.hpp:146-154)                  */
};

typedef struct ckg_out {
  int32_t max_per_track;   /* capacity of the per-track CSR rows          */
  int32_t* seq_offsets;    /* [n+1]                                        */
  int32_t* seq_surfaces;   /* [n*max_per_track]                            */
  int32_t* meas_offsets;   /* [n+1]                                        */
  int32_t* meas_surfaces;  /* [n*max_per_track]                            */
  double* meas_values;     /* [n*max_per_track*2]                          */
  double* meas_cov;        /* [n*max_per_track*4]                          */
  double* start_params;    /* [n*6]                                        */
  double* start_cov;       /* [n*36]                                       */
  double* start_frames;    /* [n*12]                                       */
  float* particle;         /* [n*2]                                        */
  int32_t* particle_pdg;   /* [n]                                          */
  double* truth_meas;      /* [n*max_per_track*6] true bound pars at each
                              measurement (may be NULL)                    */
  uint8_t* meas_outlier;   /* [n*max_per_track] 1 = displaced (may be NULL) */
  double* truth_start;     /* [n*6] true start parameters (may be NULL)    */
  int32_t* meas_subspace;  /* [n*max_per_track] CK_MEAS_* (may be NULL)    */
} ckg_out;

/* Surface table of a preset; returns the number of surfaces written
 * (at most `cap`). */
int32_t ckg_geometry(int32_t preset, ck_surface* out, int32_t cap);

/* Field of a preset. For the grid preset `values` must hold
 * ckg_field_values(preset) floats; the returned ck_field points to it. */
int64_t ckg_field_values(int32_t preset);
void ckg_field(int32_t preset, float* values, ck_field* out, int32_t n_threads);

/* Generates tracks [first_track, first_track + n_tracks) of a preset into
 * `out` (compact CSR). Returns the number of measurements written, or -1 on
 * bad arguments. */
int64_t ckg_generate(int32_t preset, uint64_t seed, int64_t first_track, int32_t n_tracks,
                     const ck_surface* surfaces, int32_t n_surfaces, const ck_field* field,
                     int32_t n_threads, ckg_out* out);

/* Poisson-distributed track counts for `n_events` events of the uneven
 * preset (mean `mean`), or log-uniform counts in [lo, hi] for the serving
 * preset (mean < 0). */
void ckg_event_sizes(uint64_t seed, int32_t n_events, double mean, int32_t lo, int32_t hi,
                     int32_t* sizes);

#ifdef __cplusplus
}
#endif

#endif /* CKGEN_H */

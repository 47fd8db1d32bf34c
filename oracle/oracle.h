/* oracle.h -- CPU restatement of SixTrackLib's element-by-element tracking.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA engine is checked
 * against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it; the product library never links, calls or falls back to it.
 *
 * Parity pin: oracle/build_ref.sh compiles the reference's own header-only
 * tracking code (sixtracklib/common/track/track.h and the be_* maps) into
 * oracle/_ref/libstref.so; tests/test_oracle_vs_ref.py checks this oracle
 * against it bit for bit, and tests/golden/ holds fixtures generated from it
 * (tests/golden/make_golden.py) plus the reference's shipped golden files.
 *
 * Particle data is the canonical "column block": 21 columns of n 8-byte
 * words in NS(Particles) field order (sixtracklib/common/particles.h:38-67):
 *   0 q0  1 mass0  2 beta0  3 gamma0  4 p0c  5 s  6 x  7 y  8 px  9 py
 *   10 zeta  11 psigma  12 delta  13 rpp  14 rvv  15 chi  16 charge_ratio
 *   17 particle_id  18 at_element  19 at_turn  20 state     (17-20: int64)
 * The lattice is a CObjects buffer image (any stored base address).
 */
#ifndef STG_ORACLE_H
#define STG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Elem-by-elem store configuration, field meaning as NS(ElemByElemConfig)
 * (sixtracklib/common/output/elem_by_elem_config.h:39-54). */
typedef struct orc_ebe_config {
    int64_t order;
    int64_t num_particles_to_store;
    int64_t num_elements_to_store;
    int64_t num_turns_to_store;
    int64_t min_particle_id;
    int64_t min_element_id;
    int64_t min_turn;
    int64_t max_particle_id;
    int64_t max_element_id;
    int64_t max_turn;
    int64_t is_rolling;
} orc_ebe_config;

/* Output columns for BeamMonitors, in lattice order of the monitors with a
 * non-zero out_address.  cols[k] is a column block of caps[k] records. */
typedef struct orc_monitor_outputs {
    int64_t num;
    void **cols;
    int64_t *caps;
} orc_monitor_outputs;

/* Global aperture mode after Drift/DriftExact: 2 always, 1 conditional on
 * length >= min_length, 0 never (SIXTRL_APERTURE_CHECK_AT_DRIFT). */
/* Host threads of the particle loops; returns the number in use. */
int orc_set_num_threads(int n);

void orc_set_aperture_mode(int mode, double min_length, double x_limit,
                           double y_limit);

/* Feature flags of the maps, as SIXTRL_TRACK_BEAMBEAM4D / _BEAMBEAM6D /
 * _SPACECHARGE / _TRICUB: 2 enabled, 1 skip, 0 disabled (defaults 2, 2, 2,
 * 0 as the reference's default build). */
void orc_set_track_flags(int bb4d, int bb6d, int sc, int tricub);

/* The 64 tricubic coefficients of one cell from its 64 corner values
 * (NS(tricub_construct_coefs), be_tricub/coefficients.h). */
void orc_tricub_coefs(const double *b, double *coefs);

int32_t orc_track_until(const uint8_t *lattice, void *cols, int64_t n,
                        int64_t idx_begin, int64_t idx_end, int64_t until_turn,
                        const orc_monitor_outputs *mon);

int32_t orc_track_line(const uint8_t *lattice, void *cols, int64_t n,
                       int64_t idx_begin, int64_t idx_end, uint64_t line_begin,
                       uint64_t line_end, int finish_turn,
                       const orc_monitor_outputs *mon);

int32_t orc_track_elem_by_elem(const uint8_t *lattice, void *cols, int64_t n,
                               int64_t idx_begin, int64_t idx_end,
                               const orc_ebe_config *cfg, void *out_cols,
                               int64_t out_n, int64_t until_turn,
                               const orc_monitor_outputs *mon);

int64_t orc_ebe_store_index(const orc_ebe_config *cfg, int64_t particle_id,
                            int64_t at_element, int64_t at_turn);

void orc_cerrf(double re, double im, double *w_re, double *w_im);
void orc_cerrf_n(const double *re, const double *im, double *w_re, double *w_im, int64_t n);

void orc_fields_gauss(double x, double y, double sigma_x, double sigma_y,
                      double min_sigma_diff, int skip_gs, double *ex,
                      double *ey, double *gx, double *gy);

int64_t orc_num_objects(const uint8_t *lattice);

#ifdef __cplusplus
}
#endif
#endif

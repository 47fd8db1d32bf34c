/* sixtracklib_gb300.h -- C ABI of the GB300-native tracking engine.
 *
 * A drop-in for the tracking hot path of SixTrackLib: the same `st_`-prefixed
 * entry points, the same CObjects buffer encoding of lattices and particle
 * sets, the same NS(Particles) SoA with state / at_turn / at_element_id
 * bookkeeping and the same int32 status convention (0 success, -1 failure,
 * OR-accumulated over particles).  Every tracking call runs on the GPU;
 * there is no CPU fallback: without a usable CUDA device the calls return
 * failure and report the reason through st_last_error().
 *
 * Each declaration names the reference interface it replaces (file:line in
 * the SixTrackLib tree).  Only plain C types cross this boundary.
 */
#ifndef SIXTRACKLIB_GB300_H
#define SIXTRACKLIB_GB300_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------- types */
/* sixtracklib/common/definitions.h, track/definitions.h:12-24 */
typedef int32_t st_track_status_t;
typedef uint64_t st_buffer_size_t;
typedef uint64_t st_buffer_addr_t;
typedef uint64_t st_object_type_id_t;
typedef int64_t st_particle_index_t;
typedef int64_t st_particle_num_elements_t;
typedef double st_particle_real_t;

#define ST_TRACK_SUCCESS 0
#define ST_TRACK_STATUS_GENERAL_FAILURE (-1)

/* object type ids: sixtracklib/common/internal/objects_type_id.h:16-55 */
#define ST_OBJECT_TYPE_PARTICLE 1
#define ST_OBJECT_TYPE_DRIFT 2
#define ST_OBJECT_TYPE_DRIFT_EXACT 3
#define ST_OBJECT_TYPE_MULTIPOLE 4
#define ST_OBJECT_TYPE_CAVITY 5
#define ST_OBJECT_TYPE_XYSHIFT 6
#define ST_OBJECT_TYPE_SROTATION 7
#define ST_OBJECT_TYPE_BEAM_BEAM_4D 8
#define ST_OBJECT_TYPE_BEAM_BEAM_6D 9
#define ST_OBJECT_TYPE_BEAM_MONITOR 10
#define ST_OBJECT_TYPE_LIMIT_RECT 11
#define ST_OBJECT_TYPE_LIMIT_ELLIPSE 12
#define ST_OBJECT_TYPE_SC_COASTING 13
#define ST_OBJECT_TYPE_SC_QGAUSSIAN_PROF 14
#define ST_OBJECT_TYPE_LIMIT_RECT_ELLIPSE 16
#define ST_OBJECT_TYPE_DIPEDGE 24
#define ST_OBJECT_TYPE_RF_MULTIPOLE 256
#define ST_OBJECT_TYPE_SC_INTERPOLATED_PROF 257
#define ST_OBJECT_TYPE_LINE_DENSITY_PROF_DATA 258
#define ST_OBJECT_TYPE_TRICUB_DATA 260
#define ST_OBJECT_TYPE_TRICUB 261
#define ST_OBJECT_TYPE_ELEM_BY_ELEM_CONF 65534

/* NS(Object): sixtracklib/common/buffer/buffer_object.h:24-30 */
typedef struct st_Object {
    st_buffer_addr_t begin_addr;
    st_object_type_id_t type_id;
    st_buffer_size_t size;
} st_Object;

/* NS(Particles): sixtracklib/common/particles.h:38-67 */
typedef struct st_Particles {
    int64_t num_particles;
    double *q0, *mass0, *beta0, *gamma0, *p0c;
    double *s, *x, *y, *px, *py, *zeta;
    double *psigma, *delta, *rpp, *rvv, *chi, *charge_ratio;
    int64_t *particle_id, *at_element_id, *at_turn, *state;
} st_Particles;

/* Beam-element structs, byte-identical to the reference's
 * (sixtracklib/common/be_<kind>/be_<kind>.h). */
typedef struct st_Drift { double length; } st_Drift;             /* be_drift.h:28-31 */
typedef struct st_DriftExact { double length; } st_DriftExact;   /* be_drift.h:159-162 */
typedef struct st_Multipole {                                    /* be_multipole.h:27-34 */
    int64_t order;
    double length, hxl, hyl;
    st_buffer_addr_t bal_addr;
} st_Multipole;
typedef struct st_RFMultipole {                                  /* be_rfmultipole.h */
    int64_t order;
    double voltage, frequency, lag;
    st_buffer_addr_t bal_addr, phase_addr;
} st_RFMultipole;
typedef struct st_Cavity { double voltage, frequency, lag; } st_Cavity; /* be_cavity.h:27-32 */
typedef struct st_XYShift { double dx, dy; } st_XYShift;         /* be_xyshift.h:26-30 */
typedef struct st_SRotation { double cos_z, sin_z; } st_SRotation; /* be_srotation.h:26-30 */
typedef struct st_LimitRect { double min_x, max_x, min_y, max_y; } st_LimitRect;
typedef struct st_LimitEllipse { double a_squ, b_squ, a_b_squ; } st_LimitEllipse;
typedef struct st_LimitRectEllipse {
    double max_x, max_y, a_squ, b_squ, a_squ_b_squ;
} st_LimitRectEllipse;
typedef struct st_DipoleEdge { double r21, r43; } st_DipoleEdge; /* be_dipedge.h */
typedef struct st_BeamMonitor {                                  /* be_monitor.h:35-45 */
    int64_t num_stores, start, skip;
    st_buffer_addr_t out_address;
    int64_t max_particle_id, min_particle_id;
    int64_t is_rolling, is_turn_ordered;
} st_BeamMonitor;
typedef struct st_BeamBeam4D { uint64_t data_size; st_buffer_addr_t data_addr; } st_BeamBeam4D;
typedef struct st_BeamBeam6D { uint64_t data_size; st_buffer_addr_t data_addr; } st_BeamBeam6D;
typedef struct st_SCCoasting {                                   /* be_beamfields.h:418-429 */
    double number_of_particles, circumference, sigma_x, sigma_y, length;
    double x_co, y_co, min_sigma_diff;
    uint64_t enabled;
} st_SCCoasting;
typedef struct st_SCQGaussProfile {                              /* be_beamfields.h:638-651 */
    double number_of_particles, bunchlength_rms, sigma_x, sigma_y, length;
    double x_co, y_co, min_sigma_diff, q_param, cq;
    uint64_t enabled;
} st_SCQGaussProfile;

/* NS(ElemByElemConfig): output/elem_by_elem_config.h:39-54 */
typedef struct st_ElemByElemConfig {
    int64_t order;
    int64_t num_particles_to_store, num_elements_to_store, num_turns_to_store;
    int64_t min_particle_id, min_element_id, min_turn;
    int64_t max_particle_id, max_element_id, max_turn;
    int64_t is_rolling;
    st_buffer_addr_t out_store_addr;
} st_ElemByElemConfig;

/* Opaque handles. */
typedef struct st_Buffer st_Buffer;
typedef struct st_TrackJob st_TrackJob;
typedef st_TrackJob st_TrackJobBase;     /* legacy name, track_job.h:139 */
typedef st_TrackJob st_TrackJobBaseNew;  /* track/track_job_base.h:53 */
typedef st_TrackJob st_CudaTrackJob;     /* cuda/track_job.h:42 */

/* ------------------------------------------------------ error reporting */
/* No reference counterpart: the last failure's reason, per thread. */
const char *st_last_error(void);

/* ------------------------------------------------------ CObjects buffer */
/* sixtracklib/common/buffer.h (NS(Buffer_new) ... NS(Buffer_delete)) */
st_Buffer *st_Buffer_new(st_buffer_size_t buffer_capacity);
st_Buffer *st_Buffer_new_from_file(const char *path);
/* Copy of an existing CObjects image (remapped to its new address). */
st_Buffer *st_Buffer_new_from_copy(const st_Buffer *other);
st_Buffer *st_Buffer_new_on_data(const unsigned char *data, st_buffer_size_t size);
void st_Buffer_delete(st_Buffer *buffer);
int32_t st_Buffer_write_to_file(const st_Buffer *buffer, const char *path);
int32_t st_Buffer_reset(st_Buffer *buffer);
/* buffer.h:263-400: sized creation, capacity management and the header
 * queries.  Objects are never freed individually, so there are no garbage
 * ranges (0); a buffer of this library lives at its stored base address,
 * so it never needs remapping (remap / refresh succeed).  Status 0 on
 * success, -1 otherwise; clear removes every object. */
st_Buffer *st_Buffer_new_detailed(st_buffer_size_t max_num_objects,
                                  st_buffer_size_t max_num_slots,
                                  st_buffer_size_t max_num_dataptrs,
                                  st_buffer_size_t max_num_garbage_ranges, uint64_t flags);
int32_t st_Buffer_reserve(st_Buffer *buffer, st_buffer_size_t max_num_objects,
                          st_buffer_size_t max_num_slots, st_buffer_size_t max_num_dataptrs,
                          st_buffer_size_t max_num_garbage_ranges);
int32_t st_Buffer_clear(st_Buffer *buffer, bool set_data_to_zero);
int32_t st_Buffer_reset_detailed(st_Buffer *buffer, st_buffer_size_t max_num_objects,
                                 st_buffer_size_t max_num_slots,
                                 st_buffer_size_t max_num_dataptrs,
                                 st_buffer_size_t max_num_garbage_ranges);
int32_t st_Buffer_reserve_capacity(st_Buffer *buffer, st_buffer_size_t capacity);
/* Replace the buffer's content with a CObjects file's. */
int32_t st_Buffer_read_from_file(st_Buffer *buffer, const char *path_to_file);
/* Write the image with its stored addresses moved to `norm_base_addr`. */
int32_t st_Buffer_write_to_file_normalized_addr(const st_Buffer *buffer, const char *path_to_file,
                                                st_buffer_addr_t norm_base_addr);
bool st_Buffer_needs_remapping(const st_Buffer *buffer);
int32_t st_Buffer_remap(st_Buffer *buffer);
int32_t st_Buffer_refresh(st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_header_size(const st_Buffer *buffer);
st_buffer_addr_t st_Buffer_get_data_end_addr(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_max_num_of_objects(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_max_num_of_slots(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_max_num_of_dataptrs(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_num_of_garbage_ranges(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_max_num_of_garbage_ranges(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_size(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_capacity(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_slot_size(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_num_of_objects(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_num_of_slots(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_num_of_dataptrs(const st_Buffer *buffer);
unsigned char *st_Buffer_get_data_begin(st_Buffer *buffer);
const unsigned char *st_Buffer_get_const_data_begin(const st_Buffer *buffer);
st_buffer_addr_t st_Buffer_get_data_begin_addr(const st_Buffer *buffer);
st_Object *st_Buffer_get_objects_begin(st_Buffer *buffer);
st_Object *st_Buffer_get_objects_end(st_Buffer *buffer);
const st_Object *st_Buffer_get_const_objects_begin(const st_Buffer *buffer);
const st_Object *st_Buffer_get_const_objects_end(const st_Buffer *buffer);
const st_Object *st_Buffer_get_const_object(const st_Buffer *buffer, st_buffer_size_t index);
st_Object *st_Buffer_get_object(st_Buffer *buffer, st_buffer_size_t index);
/* Generic object append: struct bytes plus float64/int64 arrays the given
 * pointer fields (by 8-byte word index in the struct) reference. */
void *st_Buffer_add_object(st_Buffer *buffer, const void *struct_data,
                           st_buffer_size_t struct_size, st_object_type_id_t type_id,
                           st_buffer_size_t num_dataptrs, const st_buffer_size_t *field_word_index,
                           const void *const *array_data, const st_buffer_size_t *array_words);
st_object_type_id_t st_Object_get_type_id(const st_Object *obj);
st_buffer_addr_t st_Object_get_begin_addr(const st_Object *obj);
st_buffer_size_t st_Object_get_size(const st_Object *obj);

/* ------------------------------------------------------- beam elements */
/* be_drift/be_drift.h, be_multipole/be_multipole.h, ... (NS(X_new),
 * NS(X_add), NS(X_type_id)) */
st_Drift *st_Drift_new(st_Buffer *buffer);
st_Drift *st_Drift_add(st_Buffer *buffer, double length);
st_DriftExact *st_DriftExact_new(st_Buffer *buffer);
st_DriftExact *st_DriftExact_add(st_Buffer *buffer, double length);
st_Multipole *st_Multipole_new(st_Buffer *buffer, int64_t order);
st_Multipole *st_Multipole_add(st_Buffer *buffer, int64_t order, const double *bal,
                               double length, double hxl, double hyl);
double *st_Multipole_bal(st_Multipole *mp);
st_RFMultipole *st_RFMultipole_new(st_Buffer *buffer, int64_t order);
st_RFMultipole *st_RFMultipole_add(st_Buffer *buffer, int64_t order, double voltage,
                                   double frequency, double lag, const double *bal,
                                   const double *phase);
st_Cavity *st_Cavity_new(st_Buffer *buffer);
st_Cavity *st_Cavity_add(st_Buffer *buffer, double voltage, double frequency, double lag);
st_XYShift *st_XYShift_new(st_Buffer *buffer);
st_XYShift *st_XYShift_add(st_Buffer *buffer, double dx, double dy);
st_SRotation *st_SRotation_new(st_Buffer *buffer);
st_SRotation *st_SRotation_add(st_Buffer *buffer, double angle_rad);
st_SRotation *st_SRotation_add_detailed(st_Buffer *buffer, double cos_z, double sin_z);
st_LimitRect *st_LimitRect_new(st_Buffer *buffer);
st_LimitRect *st_LimitRect_add(st_Buffer *buffer, double min_x, double max_x,
                               double min_y, double max_y);
st_LimitEllipse *st_LimitEllipse_new(st_Buffer *buffer);
st_LimitEllipse *st_LimitEllipse_add(st_Buffer *buffer, double x_half_axis,
                                     double y_half_axis);
st_LimitRectEllipse *st_LimitRectEllipse_new(st_Buffer *buffer);
st_LimitRectEllipse *st_LimitRectEllipse_add(st_Buffer *buffer, double max_x, double max_y,
                                             double a_squ, double b_squ);
st_DipoleEdge *st_DipoleEdge_new(st_Buffer *buffer);
st_DipoleEdge *st_DipoleEdge_add(st_Buffer *buffer, double r21, double r43);
st_BeamMonitor *st_BeamMonitor_new(st_Buffer *buffer);
st_BeamMonitor *st_BeamMonitor_add(st_Buffer *buffer, int64_t num_stores, int64_t start,
                                   int64_t skip, st_buffer_addr_t out_address,
                                   int64_t min_particle_id, int64_t max_particle_id,
                                   bool is_rolling, bool is_turn_ordered);
st_BeamBeam4D *st_BeamBeam4D_new(st_Buffer *buffer, st_buffer_size_t data_size);
st_BeamBeam4D *st_BeamBeam4D_add(st_Buffer *buffer, st_buffer_size_t data_size,
                                 const double *data);
st_BeamBeam6D *st_BeamBeam6D_new(st_Buffer *buffer, st_buffer_size_t data_size);
st_BeamBeam6D *st_BeamBeam6D_add(st_Buffer *buffer, st_buffer_size_t data_size,
                                 const double *data);
st_SCCoasting *st_SCCoasting_new(st_Buffer *buffer);
st_SCCoasting *st_SCCoasting_add(st_Buffer *buffer, double number_of_particles,
                                 double circumference, double sigma_x, double sigma_y,
                                 double length, double x_co, double y_co,
                                 double min_sigma_diff, bool enabled);
st_SCQGaussProfile *st_SCQGaussProfile_new(st_Buffer *buffer);
st_SCQGaussProfile *st_SCQGaussProfile_add(st_Buffer *buffer, double number_of_particles,
                                           double bunchlength_rms, double sigma_x,
                                           double sigma_y, double length, double x_co,
                                           double y_co, double min_sigma_diff,
                                           double q_param, bool enabled);

/* ------------------------------------------------------------ particles */
/* particles.h:152-170 (NS(Particles_new)), NS(Particles_buffer_get_particles),
 * NS(Particles_managed_buffer_get_particles) */
st_Particles *st_Particles_new(st_Buffer *buffer, st_buffer_size_t num_particles);
st_Particles *st_Particles_add_copy(st_Buffer *buffer, const st_Particles *orig);
st_Particles *st_Particles_buffer_get_particles(st_Buffer *buffer, st_buffer_size_t index);
const st_Particles *st_Particles_buffer_get_const_particles(const st_Buffer *buffer,
                                                            st_buffer_size_t index);
int64_t st_Particles_get_num_of_particles(const st_Particles *p);
st_buffer_size_t st_Particles_buffer_get_num_of_particle_blocks(const st_Buffer *buffer);
/* Reference momentum helpers (particles.h NS(Particles_update_delta_value),
 * NS(Particles_set_...)): beta0/gamma0 from p0c, delta-dependent columns. */
void st_Particles_set_reference(st_Particles *p, double p0c, double mass0, double q0);
void st_Particles_update_delta_value(st_Particles *p, int64_t index, double delta);
int32_t st_Particles_copy(st_Particles *dest, const st_Particles *src);

/* ----------------------------------------------------- free tracking calls */
/* common/track/track.h:86-132; each call uploads the particle set to the
 * GPU, tracks there and writes the result back into the caller's columns. */
st_track_status_t st_Track_particle_until_turn(st_Particles *particles, int64_t index,
                                               const st_Buffer *beam_elements,
                                               int64_t until_turn);
st_track_status_t st_Track_all_particles_until_turn(st_Particles *particles,
                                                    const st_Buffer *beam_elements,
                                                    int64_t until_turn);
st_track_status_t st_Track_particle_element_by_element_until_turn(
    st_Particles *particles, int64_t index, const st_ElemByElemConfig *config,
    const st_Buffer *beam_elements, int64_t until_turn);
st_track_status_t st_Track_all_particles_element_by_element_until_turn(
    st_Particles *particles, const st_ElemByElemConfig *config,
    const st_Buffer *beam_elements, int64_t until_turn);
st_track_status_t st_Track_particle_line(st_Particles *particles, int64_t index,
                                         const st_Buffer *beam_elements,
                                         st_buffer_size_t line_begin_idx,
                                         st_buffer_size_t line_end_idx, bool finish_turn);
st_track_status_t st_Track_all_particles_line(st_Particles *particles,
                                              const st_Buffer *beam_elements,
                                              st_buffer_size_t line_begin_idx,
                                              st_buffer_size_t line_end_idx,
                                              bool finish_turn);

/* Elem-by-elem configuration (output/elem_by_elem_config.h:667-763). */
int32_t st_ElemByElemConfig_init_detailed(st_ElemByElemConfig *config, int64_t order,
                                          int64_t min_particle_id, int64_t max_particle_id,
                                          int64_t min_element_id, int64_t max_element_id,
                                          int64_t min_turn, int64_t max_turn,
                                          bool is_rolling);
int64_t st_ElemByElemConfig_get_particles_store_index_details(
    const st_ElemByElemConfig *config, int64_t particle_id, int64_t at_element,
    int64_t at_turn);
int64_t st_ElemByElemConfig_get_stored_num_particles(const st_ElemByElemConfig *config);

/* ------------------------------------------------------ output buffer */
/* Host-side planning of the tracking output (output/output_buffer.h:42-260,
 * be_monitor/output_buffer.h:20-135, output/elem_by_elem_output_buffer.h,
 * output/elem_by_elem_config.c:366-375).  The particle-id / element-id /
 * turn ranges come from the particles (ids by magnitude) and from the
 * lattice's beam elements; the output holds the elem-by-elem Particles block
 * first (when until_turn_elem_by_elem exceeds the first turn), then one
 * block of (max_id - min_id + 1) * num_stores particles per beam monitor
 * that starts at or after the first turn.  Flags: 0x01 elem-by-elem,
 * 0x02 beam monitors.  Status 0 on success, -1 otherwise; slot_size must
 * be 8.  With particle ids >= 0 and a lattice of beam elements only, a
 * TrackJob's output buffer has this layout too. */
bool st_OutputBuffer_requires_output_buffer_ext(uint32_t flags);
bool st_OutputBuffer_requires_elem_by_elem_output_ext(uint32_t flags);
bool st_OutputBuffer_requires_beam_monitor_output_ext(uint32_t flags);
uint32_t st_OutputBuffer_required_for_tracking(const st_Particles *particles,
                                               const st_Buffer *beam_elements,
                                               st_buffer_size_t until_turn_elem_by_elem);
uint32_t st_OutputBuffer_required_for_tracking_of_particle_sets(
    const st_Buffer *particles_buffer, st_buffer_size_t num_particle_sets,
    const st_buffer_size_t *particle_set_indices, const st_Buffer *beam_elements,
    st_buffer_size_t until_turn_elem_by_elem);
uint32_t st_OutputBuffer_required_for_tracking_detailed(
    const st_Buffer *beam_elements, int64_t min_particle_id, int64_t max_particle_id,
    int64_t min_element_id, int64_t max_element_id, int64_t min_turn_id, int64_t max_turn_id,
    st_buffer_size_t until_turn_elem_by_elem);
int32_t st_OutputBuffer_prepare(st_Buffer *beam_elements, st_Buffer *output_buffer,
                                const st_Particles *particles,
                                st_buffer_size_t until_turn_elem_by_elem,
                                st_buffer_size_t *elem_by_elem_out_index_offset,
                                st_buffer_size_t *beam_monitor_out_index_offset,
                                int64_t *min_turn_id);
int32_t st_OutputBuffer_prepare_for_particle_sets(
    st_Buffer *beam_elements, st_Buffer *output_buffer, const st_Buffer *particles_buffer,
    st_buffer_size_t num_particle_sets, const st_buffer_size_t *particle_set_indices,
    st_buffer_size_t until_turn_elem_by_elem, st_buffer_size_t *elem_by_elem_out_index_offset,
    st_buffer_size_t *beam_monitor_out_index_offset, int64_t *min_turn_id);
int32_t st_OutputBuffer_prepare_detailed(
    st_Buffer *beam_elements, st_Buffer *output_buffer, int64_t min_particle_id,
    int64_t max_particle_id, int64_t min_element_id, int64_t max_element_id,
    int64_t min_turn_id, int64_t max_turn_id, st_buffer_size_t until_turn_elem_by_elem,
    st_buffer_size_t *elem_by_elem_out_index_offset,
    st_buffer_size_t *beam_monitor_out_index_offset, int64_t *max_elem_by_elem_turn_id);
int32_t st_OutputBuffer_calculate_output_buffer_params(
    const st_Buffer *beam_elements, const st_Particles *particles,
    st_buffer_size_t until_turn_elem_by_elem, st_buffer_size_t *num_objects,
    st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs, st_buffer_size_t *num_garbage,
    st_buffer_size_t slot_size);
int32_t st_OutputBuffer_calculate_output_buffer_params_for_particles_sets(
    const st_Buffer *beam_elements, const st_Buffer *particles_buffer,
    st_buffer_size_t num_particle_sets, const st_buffer_size_t *particle_set_indices,
    st_buffer_size_t until_turn_elem_by_elem, st_buffer_size_t *num_objects,
    st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs, st_buffer_size_t *num_garbage,
    st_buffer_size_t slot_size);
int32_t st_OutputBuffer_calculate_output_buffer_params_detailed(
    const st_Buffer *beam_elements, int64_t min_particle_id, int64_t max_particle_id,
    int64_t min_element_id, int64_t max_element_id, int64_t min_turn_id, int64_t max_turn_id,
    st_buffer_size_t until_turn_elem_by_elem, st_buffer_size_t *num_objects,
    st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs, st_buffer_size_t *num_garbage,
    st_buffer_size_t slot_size);
/* be_monitor/output_buffer.h:20-135.  assign_output_buffer points every
 * storing monitor at its block: from object 1 when an elem-by-elem block
 * precedes them, else from object 0. */
int32_t st_BeamMonitor_calculate_output_buffer_params(
    const st_Buffer *beam_elements, const st_Particles *particles,
    st_buffer_size_t *num_objects, st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs,
    st_buffer_size_t *num_garbage, st_buffer_size_t slot_size);
int32_t st_BeamMonitor_calculate_output_buffer_params_detailed(
    const st_Buffer *beam_elements, int64_t min_particle_id, int64_t max_particle_id,
    int64_t min_turn_id, st_buffer_size_t *num_objects, st_buffer_size_t *num_slots,
    st_buffer_size_t *num_dataptrs, st_buffer_size_t *num_garbage, st_buffer_size_t slot_size);
int32_t st_BeamMonitor_prepare_output_buffer(st_Buffer *beam_elements, st_Buffer *output_buffer,
                                             const st_Particles *particles,
                                             st_buffer_size_t *out_index_offset);
int32_t st_BeamMonitor_prepare_output_buffer_detailed(st_Buffer *beam_elements,
                                                      st_Buffer *output_buffer,
                                                      int64_t min_particle_id,
                                                      int64_t max_particle_id,
                                                      int64_t min_turn_id,
                                                      st_buffer_size_t *out_index_offset);
int32_t st_BeamMonitor_assign_output_buffer(st_Buffer *beam_elements, st_Buffer *output_buffer,
                                            int64_t min_turn_id,
                                            st_buffer_size_t until_turn_elem_by_elem);
int32_t st_BeamMonitor_assign_output_buffer_from_offset(st_Buffer *beam_elements,
                                                        st_Buffer *output_buffer,
                                                        int64_t min_turn_id,
                                                        st_buffer_size_t out_index_offset);
int32_t st_BeamMonitor_setup_for_particles_all(st_Buffer *beam_elements,
                                               const st_Particles *particles);
/* output/elem_by_elem_output_buffer.h:24-115, elem_by_elem_config.c:366-375 */
int32_t st_ElemByElemConfig_calculate_output_buffer_params_detailed(
    int64_t min_particle_id, int64_t max_particle_id, int64_t min_element_id,
    int64_t max_element_id, int64_t min_turn_id, int64_t max_turn_id,
    st_buffer_size_t until_turn_elem_by_elem, st_buffer_size_t *num_objects,
    st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs, st_buffer_size_t *num_garbage,
    st_buffer_size_t slot_size);
int32_t st_ElemByElemConfig_prepare_output_buffer_detailed(
    st_Buffer *output_buffer, int64_t min_particle_id, int64_t max_particle_id,
    int64_t min_element_id, int64_t max_element_id, int64_t min_turn_id,
    int64_t max_elem_by_elem_turn_id, st_buffer_size_t *out_index_offset);
int32_t st_ElemByElemConfig_assign_output_buffer(st_ElemByElemConfig *config,
                                                 st_Buffer *output_buffer,
                                                 st_buffer_size_t out_index_offset);
/* Field accessors and lifecycle of the configuration (the reference's
 * "_ext" copies of output/elem_by_elem_config.h:532-1160; create / delete
 * of elem_by_elem_config.c).  clear: ids -1, counts 0, no store address;
 * preset: clear, order -1 (invalid), rolling; active: an order and
 * something to store. */
st_ElemByElemConfig *st_ElemByElemConfig_create(void);
void st_ElemByElemConfig_delete(st_ElemByElemConfig *config);
st_ElemByElemConfig *st_ElemByElemConfig_preset_ext(st_ElemByElemConfig *config);
void st_ElemByElemConfig_clear_ext(st_ElemByElemConfig *config);
bool st_ElemByElemConfig_is_active_ext(const st_ElemByElemConfig *config);
int32_t st_ElemByElemConfig_get_order_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_num_particles_to_store_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_num_elements_to_store_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_num_turns_to_store_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_out_store_num_particles_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_min_particle_id_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_max_particle_id_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_min_element_id_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_max_element_id_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_min_turn_ext(const st_ElemByElemConfig *config);
int64_t st_ElemByElemConfig_get_max_turn_ext(const st_ElemByElemConfig *config);
bool st_ElemByElemConfig_is_rolling_ext(const st_ElemByElemConfig *config);
st_buffer_addr_t st_ElemByElemConfig_get_output_store_address_ext(
    const st_ElemByElemConfig *config);
void st_ElemByElemConfig_set_order_ext(st_ElemByElemConfig *config, int64_t order);
void st_ElemByElemConfig_set_is_rolling_ext(st_ElemByElemConfig *config, bool is_rolling);
void st_ElemByElemConfig_set_output_store_address_ext(st_ElemByElemConfig *config,
                                                      st_buffer_addr_t out_address);
/* particles.h:515-562, 3121-3230: the particle count over every Particles
 * object of a buffer; diff = lhs - rhs per column (all three of one size). */
st_buffer_size_t st_Particles_buffer_get_total_num_of_particles(const st_Buffer *buffer);
void st_Particles_calculate_difference(const st_Particles *lhs, const st_Particles *rhs,
                                       st_Particles *diff);

/* ------------------------------------------------------------- TrackJob */
/* Legacy TrackJob, common/track_job.h:139-190 and
 * common/internal/track_job.cpp:47-186.  `arch` is "cuda" (also accepted:
 * "gb300", "gpu"); the reference's "cpu" / "opencl" backends are not part
 * of this engine and are rejected with NULL.  `config_str` accepts
 * whitespace-separated key=value pairs (see st_TrackJob_get_config_str):
 *   mode=exact|fast  threads_per_block=N  track_threads_per_block=N
 *   device=N  aperture=always|never|conditional  aperture_min_length=L
 *   x_limit=X  y_limit=Y
 *   track_beambeam4d=  track_beambeam6d=  track_spacecharge=  track_tricub=
 *     enabled|skip|disabled (the reference's SIXTRL_TRACK_* build flags,
 *     track/track.h:421-575: a disabled map fails and the particle is lost,
 *     a skipped one does nothing; defaults enabled, enabled, enabled,
 *     disabled as the reference's default build)
 * and the reference's TOML forms ("[cuda]\n track_threads_per_block = N",
 * "cuda.threads_per_block = N").  Block sizes are multiples of 32 up to
 * 1024, as in the reference; the tracking kernel (track_threads_per_block,
 * else threads_per_block) runs with at most 256 threads per block. */
st_TrackJob *st_TrackJob_create(const char *arch, const char *config_str);
st_TrackJob *st_TrackJob_new(const char *arch, st_Buffer *particles_buffer,
                             st_Buffer *beam_elements_buffer, const char *config_str);
st_TrackJob *st_TrackJob_new_with_output(const char *arch, st_Buffer *particles_buffer,
                                         st_Buffer *beam_elements_buffer,
                                         st_Buffer *output_buffer,
                                         st_buffer_size_t until_turn_elem_by_elem,
                                         const char *config_str);
st_TrackJob *st_TrackJob_new_detailed(const char *arch, st_Buffer *particles_buffer,
                                      st_buffer_size_t num_particle_sets,
                                      const st_buffer_size_t *particle_set_indices,
                                      st_Buffer *beam_elements_buffer,
                                      st_Buffer *output_buffer,
                                      st_buffer_size_t until_turn_elem_by_elem,
                                      const char *config_str);
bool st_TrackJob_reset(st_TrackJob *job, st_Buffer *particles_buffer,
                       st_Buffer *beam_elements_buffer, st_Buffer *output_buffer);
bool st_TrackJob_reset_with_output(st_TrackJob *job, st_Buffer *particles_buffer,
                                   st_Buffer *beam_elements_buffer, st_Buffer *output_buffer,
                                   st_buffer_size_t until_turn_elem_by_elem);
bool st_TrackJob_reset_detailed(st_TrackJob *job, st_Buffer *particles_buffer,
                                st_buffer_size_t num_particle_sets,
                                const st_buffer_size_t *particle_set_indices,
                                st_Buffer *beam_elements_buffer, st_Buffer *output_buffer,
                                st_buffer_size_t until_turn_elem_by_elem);
void st_TrackJob_delete(st_TrackJob *job);
void st_TrackJob_clear(st_TrackJob *job);
st_track_status_t st_TrackJob_track_until(st_TrackJob *job, st_buffer_size_t until_turn);
st_track_status_t st_TrackJob_track_elem_by_elem(st_TrackJob *job,
                                                 st_buffer_size_t until_turn);
st_track_status_t st_TrackJob_track_line(st_TrackJob *job, st_buffer_size_t begin_idx,
                                         st_buffer_size_t end_idx, bool finish_turn);
void st_TrackJob_collect(st_TrackJob *job);
void st_TrackJob_collect_detailed(st_TrackJob *job, uint16_t flags);
void st_TrackJob_collect_particles(st_TrackJob *job);
void st_TrackJob_collect_beam_elements(st_TrackJob *job);
void st_TrackJob_collect_output(st_TrackJob *job);
void st_TrackJob_push(st_TrackJob *job, uint16_t flags);
void st_TrackJob_push_particles(st_TrackJob *job);
void st_TrackJob_push_beam_elements(st_TrackJob *job);
void st_TrackJob_push_output(st_TrackJob *job);
void st_TrackJob_enable_collect_particles(st_TrackJob *job);
void st_TrackJob_disable_collect_particles(st_TrackJob *job);
bool st_TrackJob_is_collecting_particles(const st_TrackJob *job);
void st_TrackJob_enable_collect_beam_elements(st_TrackJob *job);
void st_TrackJob_disable_collect_beam_elements(st_TrackJob *job);
bool st_TrackJob_is_collecting_beam_elements(const st_TrackJob *job);
void st_TrackJob_enable_collect_output(st_TrackJob *job);
void st_TrackJob_disable_collect_output(st_TrackJob *job);
bool st_TrackJob_is_collecting_output(const st_TrackJob *job);
uint16_t st_TrackJob_get_collect_flags(const st_TrackJob *job);
void st_TrackJob_set_collect_flags(st_TrackJob *job, uint16_t flags);
bool st_TrackJob_requires_collecting(const st_TrackJob *job);
/* 3, SIXTRL_ARCHITECTURE_CUDA (control/definitions.h:84-86) */
int64_t st_TrackJob_get_type_id(const st_TrackJob *job);
const char *st_TrackJob_get_type_str(const st_TrackJob *job);
bool st_TrackJob_has_device_id_str(const st_TrackJob *job);
const char *st_TrackJob_get_device_id_str(const st_TrackJob *job);
bool st_TrackJob_has_config_str(const st_TrackJob *job);
const char *st_TrackJob_get_config_str(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_get_num_particle_sets(const st_TrackJob *job);
const st_buffer_size_t *st_TrackJob_get_particle_set_indices_begin(const st_TrackJob *job);
const st_buffer_size_t *st_TrackJob_get_particle_set_indices_end(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_get_particle_set_index(const st_TrackJob *job, st_buffer_size_t n);
st_buffer_size_t st_TrackJob_get_total_num_particles_in_sets(const st_TrackJob *job);
int64_t st_TrackJob_get_min_particle_id(const st_TrackJob *job);
int64_t st_TrackJob_get_max_particle_id(const st_TrackJob *job);
int64_t st_TrackJob_get_min_element_id(const st_TrackJob *job);
int64_t st_TrackJob_get_max_element_id(const st_TrackJob *job);
int64_t st_TrackJob_get_min_initial_turn_id(const st_TrackJob *job);
int64_t st_TrackJob_get_max_initial_turn_id(const st_TrackJob *job);
st_Buffer *st_TrackJob_get_particles_buffer(st_TrackJob *job);
const st_Buffer *st_TrackJob_get_const_particles_buffer(const st_TrackJob *job);
st_Buffer *st_TrackJob_get_beam_elements_buffer(st_TrackJob *job);
const st_Buffer *st_TrackJob_get_const_beam_elements_buffer(const st_TrackJob *job);
bool st_TrackJob_has_output_buffer(const st_TrackJob *job);
bool st_TrackJob_owns_output_buffer(const st_TrackJob *job);
st_Buffer *st_TrackJob_get_output_buffer(st_TrackJob *job);
const st_Buffer *st_TrackJob_get_const_output_buffer(const st_TrackJob *job);
bool st_TrackJob_has_elem_by_elem_output(const st_TrackJob *job);
bool st_TrackJob_has_beam_monitor_output(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_get_elem_by_elem_output_buffer_offset(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_get_beam_monitor_output_buffer_offset(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_get_num_elem_by_elem_turns(const st_TrackJob *job);
bool st_TrackJob_has_elem_by_elem_config(const st_TrackJob *job);
const st_ElemByElemConfig *st_TrackJob_get_elem_by_elem_config(const st_TrackJob *job);
bool st_TrackJob_is_elem_by_elem_config_rolling(const st_TrackJob *job);
bool st_TrackJob_get_default_elem_by_elem_config_rolling_flag(const st_TrackJob *job);
void st_TrackJob_set_default_elem_by_elem_config_rolling_flag(st_TrackJob *job, bool rolling);
int64_t st_TrackJob_get_elem_by_elem_config_order(const st_TrackJob *job);
bool st_TrackJob_has_beam_monitors(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_get_num_beam_monitors(const st_TrackJob *job);
const st_buffer_size_t *st_TrackJob_get_beam_monitor_indices_begin(const st_TrackJob *job);
const st_buffer_size_t *st_TrackJob_get_beam_monitor_indices_end(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_get_beam_monitor_index(const st_TrackJob *job, st_buffer_size_t n);

/* TrackJobNew / CudaTrackJob names (track/track_job_base.h:53-65,
 * cuda/track_job.h:42-66): the same job object. */
st_CudaTrackJob *st_CudaTrackJob_create(void);
st_CudaTrackJob *st_CudaTrackJob_new_from_config_str(const char *config_str);
st_CudaTrackJob *st_CudaTrackJob_new(const char *node_id_str, st_Buffer *particles_buffer,
                                     st_Buffer *beam_elements_buffer);
st_CudaTrackJob *st_CudaTrackJob_new_with_output(const char *node_id_str,
                                                 st_Buffer *particles_buffer,
                                                 st_Buffer *beam_elements_buffer,
                                                 st_Buffer *output_buffer,
                                                 st_buffer_size_t until_turn_elem_by_elem);
st_CudaTrackJob *st_CudaTrackJob_new_detailed(const char *node_id_str,
                                              st_Buffer *particles_buffer,
                                              st_buffer_size_t num_particle_sets,
                                              const st_buffer_size_t *particle_set_indices,
                                              st_Buffer *beam_elements_buffer,
                                              st_Buffer *output_buffer,
                                              st_buffer_size_t until_turn_elem_by_elem,
                                              const char *config_str);
void st_TrackJobNew_delete(st_TrackJobBaseNew *job);
st_track_status_t st_TrackJobNew_track_until(st_TrackJobBaseNew *job, st_buffer_size_t until_turn);
st_track_status_t st_TrackJobNew_track_elem_by_elem(st_TrackJobBaseNew *job,
                                                    st_buffer_size_t until_turn);
st_track_status_t st_TrackJobNew_track_line(st_TrackJobBaseNew *job, st_buffer_size_t begin_idx,
                                            st_buffer_size_t end_idx, bool finish_turn);
int32_t st_TrackJobNew_collect_particles(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_collect_beam_elements(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_collect_output(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_collect(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_push_particles(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_push_beam_elements(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_push_output(st_TrackJobBaseNew *job);
/* Debug mode (track/track_job_base.h:182-189, the CUDA job's debug
 * kernels track/track_kernel_impl.h:149-250).  In debug mode every
 * tracking call first validates its inputs and records the outcome in a
 * debug register: flags from bit 32 up as the reference numbers them (2^32
 * particle index, 2^33 particle buffer null, 2^34 beam-element buffer null,
 * 2^36 particle-set index, 2^37 / 2^38 particle / beam-element buffer needs
 * remapping, 2^39 line boundaries, 2^40 until_turn), then the engine's own
 * (2^41 a shared-memory pipeline wait timed out, 2^42 elem-by-elem tracking
 * without an elem-by-elem output), and the track status in the low 32 bits
 * (control/debug_register.h:59-80).  A raised flag makes the call return
 * -1 without tracking.  enable / disable return 0 (-1 for a null job);
 * collect_debug_flag returns 0 in debug mode (the register lives on the
 * host).  st_TrackJobNew_get_debug_register has no counterpart in the
 * reference (which keeps its register inside the job): it returns it. */
bool st_TrackJobNew_is_in_debug_mode(const st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_enable_debug_mode(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_disable_debug_mode(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_collect_debug_flag(st_TrackJobBaseNew *job);
uint64_t st_TrackJobNew_get_debug_register(const st_TrackJobBaseNew *job);
/* Stored buffers and address assignment (common/track_job.h: stored
 * buffers, NS(AssignAddressItem) of buffer/assign_address_item.h).  A stored
 * buffer is a caller's st_Buffer kept by the job under an id >= 1024.  With
 * take_ownership its contents move into a buffer of the job's (object
 * addresses unchanged; st_TrackJob_stored_buffer returns the new handle),
 * the caller's buffer is left empty and is deleted if
 * delete_ptr_after_move; owned buffers are deleted with the job.  An item names a destination pointer field
 * (buffer id -- 2 for the beam elements, or a stored buffer --, object
 * index and type id, byte offset) and a source (buffer id -- 1 particles,
 * 2 beam elements or a stored buffer --, object index and type id, byte
 * offset); assigning writes the source object's address plus its offset
 * into the field, after the reference's checks (type ids, sizes, 8-byte
 * alignment), and recompiles the lattice when the beam elements changed.
 * The engine reads such an address when it compiles the lattice (an
 * SCInterpolatedProfile's line-density table), so a stored buffer must
 * live as long as the job.  Beam monitors write into the job's own output
 * buffer whatever their out_address says.  Status 0 on success, -1
 * otherwise; ids / indices are 0 on failure. */
typedef struct st_AssignAddressItem {
    uint64_t dest_buffer_id, src_buffer_id, dest_elem_type_id, src_elem_type_id;
    uint64_t dest_elem_index, src_elem_index, dest_pointer_offset, src_pointer_offset;
} st_AssignAddressItem;
st_buffer_size_t st_TrackJob_add_stored_buffer(st_TrackJob *job, st_Buffer *buffer,
                                               bool take_ownership, bool delete_ptr_after_move);
st_buffer_size_t st_TrackJob_create_stored_buffer(st_TrackJob *job,
                                                  st_buffer_size_t buffer_capacity);
int32_t st_TrackJob_remove_stored_buffer(st_TrackJob *job, st_buffer_size_t buffer_id);
bool st_TrackJob_has_stored_buffers(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_num_stored_buffers(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_min_stored_buffer_id(const st_TrackJob *job);
st_buffer_size_t st_TrackJob_max_stored_buffer_id(const st_TrackJob *job);
bool st_TrackJob_owns_stored_buffer(const st_TrackJob *job, st_buffer_size_t buffer_id);
st_Buffer *st_TrackJob_stored_buffer(st_TrackJob *job, st_buffer_size_t buffer_id);
const st_Buffer *st_TrackJob_const_stored_buffer(const st_TrackJob *job,
                                                 st_buffer_size_t buffer_id);
int32_t st_TrackJob_push_stored_buffer(st_TrackJob *job, st_buffer_size_t buffer_id);
int32_t st_TrackJob_collect_stored_buffer(st_TrackJob *job, st_buffer_size_t buffer_id);
st_AssignAddressItem *st_TrackJob_add_assign_address_item(st_TrackJob *job,
                                                          const st_AssignAddressItem *item);
st_AssignAddressItem *st_TrackJob_add_assign_address_item_detailed(
    st_TrackJob *job, st_object_type_id_t dest_type_id, st_buffer_size_t dest_buffer_id,
    st_buffer_size_t dest_elem_index, st_buffer_size_t dest_pointer_offset,
    st_object_type_id_t src_type_id, st_buffer_size_t src_buffer_id,
    st_buffer_size_t src_elem_index, st_buffer_size_t src_pointer_offset);
bool st_TrackJob_has_assign_address_item(const st_TrackJob *job,
                                         const st_AssignAddressItem *item);
bool st_TrackJob_has_assign_item_by_index(const st_TrackJob *job, st_buffer_size_t dest_buffer_id,
                                          st_buffer_size_t src_buffer_id,
                                          st_buffer_size_t assign_item_index);
bool st_TrackJob_has_assign_items(const st_TrackJob *job, st_buffer_size_t dest_buffer_id,
                                  st_buffer_size_t src_buffer_id);
st_buffer_size_t st_TrackJob_index_of_assign_address_item(const st_TrackJob *job,
                                                          const st_AssignAddressItem *item);
st_buffer_size_t st_TrackJob_num_assign_items(const st_TrackJob *job,
                                              st_buffer_size_t dest_buffer_id,
                                              st_buffer_size_t src_buffer_id);
st_buffer_size_t st_TrackJob_total_num_assign_items(const st_TrackJob *job);
const st_AssignAddressItem *st_TrackJob_ptr_assign_address_item(
    const st_TrackJob *job, const st_AssignAddressItem *item);
const st_AssignAddressItem *st_TrackJob_ptr_assign_address_item_by_index(
    const st_TrackJob *job, st_buffer_size_t dest_buffer_id, st_buffer_size_t src_buffer_id,
    st_buffer_size_t assign_address_item_index);
int32_t st_TrackJob_commit_address_assignments(st_TrackJob *job);
int32_t st_TrackJob_assign_all_addresses(st_TrackJob *job);
int32_t st_TrackJob_assign_addresses(st_TrackJob *job, st_buffer_size_t dest_buffer_id,
                                     st_buffer_size_t src_buffer_id);

/* Device addresses of a particle set's columns
 * (particles/particles_addr.h:27-55): num_particles, then the address of
 * each of the 21 columns in NS(Particles) order. */
typedef struct st_ParticlesAddr {
    int64_t num_particles;
    uint64_t q0_addr, mass0_addr, beta0_addr, gamma0_addr, p0c_addr, s_addr, x_addr, y_addr,
        px_addr, py_addr, zeta_addr, psigma_addr, delta_addr, rpp_addr, rvv_addr, chi_addr,
        charge_ratio_addr, particle_id_addr, at_element_id_addr, at_turn_addr, state_addr;
} st_ParticlesAddr;
/* common/track_job.h:266-289 and track/track_job_base.h:150-175: the
 * device addresses of the job's particle sets, for kernels of the caller's
 * own that work on them in place.  `index` is the object index of a
 * particle set in the particles buffer; objects the job does not track
 * have no addresses (NULL).  The addresses stay valid until the job is
 * reset or deleted.  Status 0 on success, -1 otherwise. */
bool st_TrackJob_can_fetch_particles_addr(const st_TrackJob *job);
bool st_TrackJob_has_particles_addr(const st_TrackJob *job);
int32_t st_TrackJob_fetch_particle_addresses(st_TrackJob *job);
int32_t st_TrackJob_clear_particle_addresses(st_TrackJob *job, st_buffer_size_t index);
int32_t st_TrackJob_clear_all_particle_addresses(st_TrackJob *job);
const st_ParticlesAddr *st_TrackJob_particle_addresses(const st_TrackJob *job,
                                                        st_buffer_size_t index);
bool st_TrackJobNew_can_fetch_particle_addresses(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_has_particle_addresses(const st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_fetch_particle_addresses(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_clear_particle_addresses(st_TrackJobBaseNew *job,
                                                st_buffer_size_t particle_set_index);
int32_t st_TrackJobNew_clear_all_particle_addresses(st_TrackJobBaseNew *job);
const st_ParticlesAddr *st_TrackJobNew_get_particle_addresses(const st_TrackJobBaseNew *job,
                                                               st_buffer_size_t particle_set_index);
/* The rest of the TrackJobNew set that maps onto this job
 * (track/track_job_base.h:70-420): construction, reset (0 on success, -1 on
 * failure), buffers and output layout, collect / push flags. */
st_TrackJobBaseNew *st_TrackJobNew_create(const char *arch_str, const char *config_str);
st_TrackJobBaseNew *st_TrackJobNew_new(const char *arch, st_Buffer *particles_buffer,
                                       st_Buffer *beam_elements_buffer, const char *config_str);
st_TrackJobBaseNew *st_TrackJobNew_new_with_output(const char *arch, st_Buffer *particles_buffer,
                                                   st_Buffer *beam_elements_buffer,
                                                   st_Buffer *output_buffer,
                                                   st_buffer_size_t until_turn_elem_by_elem,
                                                   const char *config_str);
st_TrackJobBaseNew *st_TrackJobNew_new_detailed(const char *arch, st_Buffer *particles_buffer,
                                                st_buffer_size_t num_particle_sets,
                                                const st_buffer_size_t *particle_set_indices,
                                                st_Buffer *beam_elements_buffer,
                                                st_Buffer *output_buffer,
                                                st_buffer_size_t until_turn_elem_by_elem,
                                                const char *config_str);
int32_t st_TrackJobNew_reset(st_TrackJobBaseNew *job, st_Buffer *particles_buffer,
                             st_Buffer *beam_elements_buffer, st_Buffer *output_buffer);
int32_t st_TrackJobNew_reset_with_output(st_TrackJobBaseNew *job, st_Buffer *particles_buffer,
                                         st_Buffer *beam_elements_buffer, st_Buffer *output_buffer,
                                         st_buffer_size_t until_turn_elem_by_elem);
int32_t st_TrackJobNew_reset_detailed(st_TrackJobBaseNew *job, st_Buffer *particles_buffer,
                                      st_buffer_size_t num_particle_sets,
                                      const st_buffer_size_t *particle_set_indices,
                                      st_Buffer *beam_elements_buffer, st_Buffer *output_buffer,
                                      st_buffer_size_t until_turn_elem_by_elem);
void st_TrackJobNew_clear(st_TrackJobBaseNew *job);
uint16_t st_TrackJobNew_push(st_TrackJobBaseNew *job, uint16_t flags);
bool st_TrackJobNew_requires_collecting(const st_TrackJobBaseNew *job);
st_Buffer *st_TrackJobNew_get_particles_buffer(st_TrackJobBaseNew *job);
const st_Buffer *st_TrackJobNew_get_const_particles_buffer(const st_TrackJobBaseNew *job);
st_Buffer *st_TrackJobNew_get_beam_elements_buffer(st_TrackJobBaseNew *job);
const st_Buffer *st_TrackJobNew_get_const_beam_elements_buffer(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_has_output_buffer(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_owns_output_buffer(const st_TrackJobBaseNew *job);
st_Buffer *st_TrackJobNew_get_output_buffer(st_TrackJobBaseNew *job);
const st_Buffer *st_TrackJobNew_get_const_output_buffer(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_has_elem_by_elem_output(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_has_beam_monitor_output(const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_get_elem_by_elem_output_buffer_offset(
    const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_get_beam_monitor_output_buffer_offset(
    const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_get_num_beam_monitors(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_has_beam_monitors(const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_get_num_particle_sets(const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_get_total_num_of_particles(const st_TrackJobBaseNew *job);
const char *st_TrackJobNew_get_arch_string(const st_TrackJobBaseNew *job);
/* track/track_job_base.h: NS(TrackJobNew_get_arch_id), _has_arch_string;
 * the arch id is 3, SIXTRL_ARCHITECTURE_CUDA */
uint32_t st_TrackJobNew_get_arch_id(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_has_arch_string(const st_TrackJobBaseNew *job);
/* cuda/track_job.h:27-38: the CUDA devices this process can use (node
 * index k = CUDA device k); the index list returns how many it wrote. */
st_buffer_size_t st_CudaTrackJob_get_num_available_nodes(void);
st_buffer_size_t st_CudaTrackJob_get_available_node_indices_list(st_buffer_size_t max_num_node_indices,
                                                                 int64_t *node_indices_begin);
bool st_TrackJobNew_has_config_str(const st_TrackJobBaseNew *job);
const char *st_TrackJobNew_get_config_str(const st_TrackJobBaseNew *job);
uint16_t st_TrackJobNew_get_collect_flags(const st_TrackJobBaseNew *job);
void st_TrackJobNew_set_collect_flags(st_TrackJobBaseNew *job, uint16_t flags);
bool st_TrackJobNew_is_collecting_particles(const st_TrackJobBaseNew *job);
void st_TrackJobNew_enable_collect_particles(st_TrackJobBaseNew *job);
void st_TrackJobNew_disable_collect_particles(st_TrackJobBaseNew *job);
/* cuda/track_job.h: the tracking kernel's block size as it runs, and the
 * configured threads_per_block. */
uint64_t st_CudaTrackJob_default_track_threads_per_block(const st_CudaTrackJob *job);
uint64_t st_CudaTrackJob_default_threads_per_block(const st_CudaTrackJob *job);

/* --------------------------------------------- device-resident interface */
/* No reference counterpart: the engine's own entry points for callers that
 * keep particle columns resident on the GPU (the Python/PyTorch layer, the
 * benchmark).  `d_cols` is a device pointer to a 21 x n column block (see
 * sixtracklib_gb300/particles.py), `stream` a cudaStream_t (0 = default).
 * A compiled lattice is an engine-side device copy of a CObjects lattice. */
typedef struct st_DeviceLattice st_DeviceLattice;
st_DeviceLattice *st_DeviceLattice_new(const unsigned char *lattice_image,
                                       st_buffer_size_t image_size, const char *config_str);
void st_DeviceLattice_delete(st_DeviceLattice *lat);
int64_t st_DeviceLattice_num_elements(const st_DeviceLattice *lat);
int64_t st_DeviceLattice_num_chunks(const st_DeviceLattice *lat);
st_track_status_t st_DeviceLattice_track_until(st_DeviceLattice *lat, void *d_cols,
                                               int64_t num_particles, int64_t until_turn,
                                               void *stream);
st_track_status_t st_DeviceLattice_track_line(st_DeviceLattice *lat, void *d_cols,
                                              int64_t num_particles, uint64_t begin_idx,
                                              uint64_t end_idx, bool finish_turn,
                                              void *stream);
/* Launch without waiting for the status word (asynchronous on `stream`);
 * st_DeviceLattice_last_status() synchronises and returns it.  The
 * particle-selection scratch and the status words are shared by every call
 * on a GPU: a call that uses them waits on the GPU for the previous such
 * call's work to finish, also when it was launched on another stream (an
 * event recorded per GPU), so overlapping calls are serialised, not raced.
 * last_status() reports the status of the last call on the lattice's GPU. */
int32_t st_DeviceLattice_launch_until(st_DeviceLattice *lat, void *d_cols,
                                      int64_t num_particles, int64_t until_turn, void *stream);
st_track_status_t st_DeviceLattice_last_status(st_DeviceLattice *lat);
/* No counterpart in the reference.  Same as st_DeviceLattice_track_until,
 * for callers that must not allocate device memory while they track (code
 * inside another framework's allocator, fixed-budget real-time loops): the
 * call uses no cudaMalloc / cudaFree; its scratch is a static device array
 * sized for at most 1,048,576 particles (larger calls fail with -1).  The
 * first call on a device resolves that array's address (make it before any
 * stream capture); calls overlapping on one GPU share the array and race.
 * Synchronises `stream` and returns the track status. */
st_track_status_t st_DeviceLattice_track_until_noalloc(st_DeviceLattice *lat, void *d_cols,
                                                        int64_t num_particles,
                                                        int64_t until_turn, void *stream);

/* ------------------------------------------------------ differentiation */
/* No reference counterpart (the reference has no derivatives).  Overwrite
 * element parameters of a compiled lattice in place: for entry j,
 * kind[j] >= 0 sets multipole coefficient bal[kind[j]] of element
 * element[j] (bal[2k] = knl[k] / k!, bal[2k+1] = ksl[k] / k!, as stored in
 * the CObjects Multipole, be_multipole/be_multipole.h), kind[j] == -1 sets
 * the voltage of cavity element[j].  All entries are validated before any
 * is written; the call synchronises the device.  Host pointers. */
st_track_status_t st_DeviceLattice_set_parameters(st_DeviceLattice *lat, int64_t num,
                                                  const int64_t *element, const int32_t *kind,
                                                  const double *value);
/* No reference counterpart.  Reverse-mode derivative of turns
 * [turn_begin, turn_end) of until-turn tracking.  d_start / d_end: 21 x n
 * column blocks holding the particles at turn_begin and at turn_end (the
 * results of st_DeviceLattice_track_until to those turns).  d_lam: 6 x n
 * doubles (rows x, px, y, py, zeta, delta) holding dL/d(coordinates at
 * turn_end) on entry and dL/d(coordinates at turn_begin) on return, for the
 * particles alive at turn_begin (a particle lost inside the range has its
 * row taken as dL/d(coordinates where it was lost)); other columns are left
 * unchanged.  Intermediate turns are reconstructed by inverting the maps, so
 * the accuracy is best for short ranges (one turn: exact re-anchoring).
 * Parameter derivatives: d_param_begin[e] .. d_param_begin[e + 1] - 1 index
 * the entries of element e in d_param_kind (bal index, or -1 for a cavity
 * voltage) and d_param_id (slot of d_grad, every id < num_slots);
 * num_elements + 1 offsets; the range's contribution is added to d_grad.
 * Pass d_param_begin = NULL for coordinate derivatives only.  Every map the
 * engine tracks has an adjoint; lattices with a map compiled out (TriCub) or
 * an unknown type id are refused (-1).
 * Asynchronous on `stream`; device pointers except `lat`.  Uses the GPU's
 * shared particle-selection scratch, ordered after (and before) other calls
 * that use it as st_DeviceLattice_launch_until describes. */
st_track_status_t st_DeviceLattice_adjoint_turns(st_DeviceLattice *lat, const void *d_start,
                                                 const void *d_end, int64_t num_particles,
                                                 int64_t turn_begin, int64_t turn_end,
                                                 double *d_lam, const int32_t *d_param_begin,
                                                 const int32_t *d_param_kind,
                                                 const int32_t *d_param_id, int32_t num_slots,
                                                 double *d_grad, void *stream);
/* ------------------------------------------------------------ batching */
/* No reference counterpart (the reference tracks one lattice per job).  A
 * batch tracks many lattice variants, each with its own device-resident
 * particle block, with one persistent kernel: tiles of particles of all
 * variants, longest lattice first, are taken by the CTAs from a global
 * counter.  Results are bit-identical to st_DeviceLattice_track_until on each
 * variant alone.  All lattices must be on one device with one arithmetic mode
 * (the "mode" of their configuration).  config: threads_per_block,
 * blocks_per_sm (1 or 2), stages (2..8), turns_per_launch; all optional. */
typedef struct st_BatchTracker st_BatchTracker;
st_BatchTracker *st_BatchTracker_new(st_DeviceLattice *const *lattices, int32_t num_variants,
                                     const char *config);
void st_BatchTracker_delete(st_BatchTracker *batch);
/* One 21 x n column block per variant (device pointers; n may be 0).  The
 * lattices and blocks must outlive the batch's use of them. */
int32_t st_BatchTracker_set_particles(st_BatchTracker *batch, void *const *d_cols,
                                      const int64_t *num_particles);
/* Track every variant's particles until `until_turn`, in launches of
 * turns_per_launch turns starting at from_turn (particles already past a
 * launch's turn are left alone); synchronises `stream`, returns the status. */
st_track_status_t st_BatchTracker_track_until(st_BatchTracker *batch, int64_t from_turn,
                                              int64_t until_turn, void *stream);
/* Capture the launches that advance every variant by turns_per_replay turns
 * into a CUDA graph.  Each replay starts at the batch's turn counter (set by
 * st_BatchTracker_set_turn, asynchronous on `stream`) and advances it. */
int32_t st_BatchTracker_capture(st_BatchTracker *batch, int64_t turns_per_replay);
int32_t st_BatchTracker_set_turn(st_BatchTracker *batch, int64_t turn, void *stream);
int32_t st_BatchTracker_replay(st_BatchTracker *batch, void *stream);
/* Synchronise `stream` and return the OR of the statuses since the last
 * replay or track_until. */
st_track_status_t st_BatchTracker_status(st_BatchTracker *batch, void *stream);
int32_t st_BatchTracker_get_shape(const st_BatchTracker *batch, int32_t *threads_per_block,
                                  int32_t *blocks_per_sm, int32_t *stages,
                                  int32_t *turns_per_launch);
/* Autotuner: times launch shapes (threads per block, register tier,
 * shared-memory stages, turns per launch; coordinate descent, two passes)
 * on a copy of the first sample_fraction of every variant's particles for
 * trial_turns turns and keeps the fastest.  The batch's particles are not
 * modified; a captured graph is dropped.  *best_ms: the winning trial. */
int32_t st_BatchTracker_autotune(st_BatchTracker *batch, double sample_fraction,
                                 int64_t trial_turns, double *best_ms);

/* Kernel-launch counter (for launch accounting in benchmarks). */
uint64_t st_engine_kernel_launches(void);
/* Compile-time properties of the engine build. */
const char *st_engine_build_info(void);
/* Measured dense FP64 FMA throughput of `device` in TFLOP/s (FMA = 2 flops);
 * the denominator of the tracking kernel's roofline. */
double st_engine_measure_fp64_peak(int device);
/* The fast arithmetic policy's exponential (a table-driven e^x, within one
 * ulp) on n values of device memory x, into device memory y, on `stream` (a
 * cudaStream_t, NULL: the default stream); the CUDA error code of the
 * launch.  For checking the policy's arithmetic; the tracking maps call it
 * inline. */
int32_t st_engine_exp_fast(const double *x, double *y, int64_t n, void *stream);
/* The fast arithmetic policy's reciprocal (the hardware estimate refined by
 * one third-order step, within about one ulp of 1 / x) on n values of device
 * memory x, into device memory y, as st_engine_exp_fast. */
int32_t st_engine_rcp_fast(const double *x, double *y, int64_t n, void *stream);

#ifdef __cplusplus
}
#endif

#include "sixtracklib_gb300_aliases.h"

#endif /* SIXTRACKLIB_GB300_H */

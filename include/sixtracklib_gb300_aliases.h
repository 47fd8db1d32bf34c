/* sixtracklib_gb300_aliases.h -- the other C names under which the
 * reference's Python bindings (python/sixtracklib/stcommon.py) bind entry
 * points of this path: the "_ext" spellings of buffer, particle and
 * elem-by-elem functions (the reference's out-of-line copies of inline
 * functions) and the TrackJobNew names of TrackJob calls
 * (common/track/track_job_base.h).  Each behaves exactly as the function
 * it names without the suffix / with "TrackJob_"; the one exception is
 * st_TrackJobNew_collect_detailed, which returns the flags it collected
 * (track/track_job_base.cpp:87-90) where the legacy call returns nothing.
 * Included by sixtracklib_gb300.h. */
#ifndef SIXTRACKLIB_GB300_ALIASES_H
#define SIXTRACKLIB_GB300_ALIASES_H

#ifdef __cplusplus
extern "C" {
#endif

/* "_ext" spellings */
int32_t st_Buffer_clear_ext(st_Buffer *buffer, bool set_data_to_zero);
st_buffer_size_t st_Buffer_get_capacity_ext(const st_Buffer *buffer);
st_buffer_addr_t st_Buffer_get_data_begin_addr_ext(const st_Buffer *buffer);
st_buffer_addr_t st_Buffer_get_data_end_addr_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_header_size_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_max_num_of_dataptrs_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_max_num_of_garbage_ranges_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_max_num_of_objects_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_max_num_of_slots_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_num_of_dataptrs_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_num_of_garbage_ranges_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_num_of_objects_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_num_of_slots_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_size_ext(const st_Buffer *buffer);
st_buffer_size_t st_Buffer_get_slot_size_ext(const st_Buffer *buffer);
bool st_Buffer_needs_remapping_ext(const st_Buffer *buffer);
int32_t st_Buffer_refresh_ext(st_Buffer *buffer);
int32_t st_Buffer_remap_ext(st_Buffer *buffer);
int32_t st_Buffer_reserve_capacity_ext(st_Buffer *buffer, st_buffer_size_t capacity);
int32_t st_Buffer_reserve_ext(st_Buffer *buffer, st_buffer_size_t max_num_objects, st_buffer_size_t
    max_num_slots, st_buffer_size_t max_num_dataptrs, st_buffer_size_t max_num_garbage_ranges);
int32_t st_Buffer_reset_detailed_ext(st_Buffer *buffer, st_buffer_size_t max_num_objects,
    st_buffer_size_t max_num_slots, st_buffer_size_t max_num_dataptrs, st_buffer_size_t
    max_num_garbage_ranges);
int32_t st_Buffer_reset_ext(st_Buffer *buffer);
int64_t st_ElemByElemConfig_get_particles_store_index_details_ext( const st_ElemByElemConfig
    *config, int64_t particle_id, int64_t at_element, int64_t at_turn);
int32_t st_ElemByElemConfig_init_detailed_ext(st_ElemByElemConfig *config, int64_t order, int64_t
    min_particle_id, int64_t max_particle_id, int64_t min_element_id, int64_t max_element_id,
    int64_t min_turn, int64_t max_turn, bool is_rolling);
st_Particles *st_Particles_add_copy_ext(st_Buffer *buffer, const st_Particles *orig);
st_buffer_size_t st_Particles_buffer_get_num_of_particle_blocks_ext(const st_Buffer *buffer);
st_Particles *st_Particles_buffer_get_particles_ext(st_Buffer *buffer, st_buffer_size_t index);
st_buffer_size_t st_Particles_buffer_get_total_num_of_particles_ext(const st_Buffer *buffer);
void st_Particles_calculate_difference_ext(const st_Particles *lhs, const st_Particles *rhs,
    st_Particles *diff);
int32_t st_Particles_copy_ext(st_Particles *dest, const st_Particles *src);
int64_t st_Particles_get_num_of_particles_ext(const st_Particles *p);
st_Particles *st_Particles_new_ext(st_Buffer *buffer, st_buffer_size_t num_particles);

/* TrackJobNew names (common/track/track_job_base.h) */
uint16_t st_TrackJobNew_collect_detailed(st_TrackJobBaseNew *job, uint16_t flags);
st_AssignAddressItem *st_TrackJobNew_add_assign_address_item(st_TrackJobBaseNew *job, const
    st_AssignAddressItem *item);
st_AssignAddressItem *st_TrackJobNew_add_assign_address_item_detailed( st_TrackJobBaseNew *job,
    st_object_type_id_t dest_type_id, st_buffer_size_t dest_buffer_id, st_buffer_size_t
    dest_elem_index, st_buffer_size_t dest_pointer_offset, st_object_type_id_t src_type_id,
    st_buffer_size_t src_buffer_id, st_buffer_size_t src_elem_index, st_buffer_size_t
    src_pointer_offset);
st_buffer_size_t st_TrackJobNew_add_stored_buffer(st_TrackJobBaseNew *job, st_Buffer *buffer, bool
    take_ownership, bool delete_ptr_after_move);
int32_t st_TrackJobNew_assign_addresses(st_TrackJobBaseNew *job, st_buffer_size_t dest_buffer_id,
    st_buffer_size_t src_buffer_id);
int32_t st_TrackJobNew_assign_all_addresses(st_TrackJobBaseNew *job);
int32_t st_TrackJobNew_collect_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t buffer_id);
int32_t st_TrackJobNew_commit_address_assignments(st_TrackJobBaseNew *job);
const st_Buffer *st_TrackJobNew_const_stored_buffer(const st_TrackJobBaseNew *job, st_buffer_size_t
    buffer_id);
st_buffer_size_t st_TrackJobNew_create_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t
    buffer_capacity);
void st_TrackJobNew_disable_collect_beam_elements(st_TrackJobBaseNew *job);
void st_TrackJobNew_disable_collect_output(st_TrackJobBaseNew *job);
void st_TrackJobNew_enable_collect_beam_elements(st_TrackJobBaseNew *job);
void st_TrackJobNew_enable_collect_output(st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_get_beam_monitor_index(const st_TrackJobBaseNew *job,
    st_buffer_size_t n);
const st_buffer_size_t *st_TrackJobNew_get_beam_monitor_indices_begin(const st_TrackJobBaseNew
    *job);
const st_buffer_size_t *st_TrackJobNew_get_beam_monitor_indices_end(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_get_default_elem_by_elem_config_rolling_flag(const st_TrackJobBaseNew *job);
const st_ElemByElemConfig *st_TrackJobNew_get_elem_by_elem_config(const st_TrackJobBaseNew *job);
int64_t st_TrackJobNew_get_elem_by_elem_config_order(const st_TrackJobBaseNew *job);
int64_t st_TrackJobNew_get_max_element_id(const st_TrackJobBaseNew *job);
int64_t st_TrackJobNew_get_max_initial_turn_id(const st_TrackJobBaseNew *job);
int64_t st_TrackJobNew_get_max_particle_id(const st_TrackJobBaseNew *job);
int64_t st_TrackJobNew_get_min_element_id(const st_TrackJobBaseNew *job);
int64_t st_TrackJobNew_get_min_initial_turn_id(const st_TrackJobBaseNew *job);
int64_t st_TrackJobNew_get_min_particle_id(const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_get_num_elem_by_elem_turns(const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_get_particle_set_index(const st_TrackJobBaseNew *job,
    st_buffer_size_t n);
const st_buffer_size_t *st_TrackJobNew_get_particle_set_indices_begin(const st_TrackJobBaseNew
    *job);
const st_buffer_size_t *st_TrackJobNew_get_particle_set_indices_end(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_has_assign_address_item(const st_TrackJobBaseNew *job, const
    st_AssignAddressItem *item);
bool st_TrackJobNew_has_assign_item_by_index(const st_TrackJobBaseNew *job, st_buffer_size_t
    dest_buffer_id, st_buffer_size_t src_buffer_id, st_buffer_size_t assign_item_index);
bool st_TrackJobNew_has_assign_items(const st_TrackJobBaseNew *job, st_buffer_size_t
    dest_buffer_id, st_buffer_size_t src_buffer_id);
bool st_TrackJobNew_has_elem_by_elem_config(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_has_stored_buffers(const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_index_of_assign_address_item(const st_TrackJobBaseNew *job, const
    st_AssignAddressItem *item);
bool st_TrackJobNew_is_collecting_beam_elements(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_is_collecting_output(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_is_elem_by_elem_config_rolling(const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_max_stored_buffer_id(const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_min_stored_buffer_id(const st_TrackJobBaseNew *job);
st_buffer_size_t st_TrackJobNew_num_assign_items(const st_TrackJobBaseNew *job, st_buffer_size_t
    dest_buffer_id, st_buffer_size_t src_buffer_id);
st_buffer_size_t st_TrackJobNew_num_stored_buffers(const st_TrackJobBaseNew *job);
bool st_TrackJobNew_owns_stored_buffer(const st_TrackJobBaseNew *job, st_buffer_size_t buffer_id);
const st_AssignAddressItem *st_TrackJobNew_ptr_assign_address_item( const st_TrackJobBaseNew *job,
    const st_AssignAddressItem *item);
const st_AssignAddressItem *st_TrackJobNew_ptr_assign_address_item_by_index( const
    st_TrackJobBaseNew *job, st_buffer_size_t dest_buffer_id, st_buffer_size_t src_buffer_id,
    st_buffer_size_t assign_address_item_index);
int32_t st_TrackJobNew_push_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t buffer_id);
int32_t st_TrackJobNew_remove_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t buffer_id);
void st_TrackJobNew_set_default_elem_by_elem_config_rolling_flag(st_TrackJobBaseNew *job, bool
    rolling);
st_Buffer *st_TrackJobNew_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t buffer_id);
st_buffer_size_t st_TrackJobNew_total_num_assign_items(const st_TrackJobBaseNew *job);

/* The legacy TrackJob's names for the particle-address calls
 * (common/track_job.h:478-492) */
int32_t st_TrackJob_fetch_particles_addr(st_TrackJob *job);
int32_t st_TrackJob_clear_particles_addr(st_TrackJob *job, st_buffer_size_t index);
int32_t st_TrackJob_clear_all_particles_addr(st_TrackJob *job);
const st_ParticlesAddr *st_TrackJob_particles_addr(const st_TrackJob *job,
                                                   st_buffer_size_t index);

#ifdef __cplusplus
}
#endif
#endif

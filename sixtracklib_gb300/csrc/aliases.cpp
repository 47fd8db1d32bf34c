// aliases.cpp -- the reference's other C names for entry points of this
// library (declared in sixtracklib_gb300_aliases.h): each forwards to the
// function it names.
#include "common.h"

extern "C" {

// "_ext" spellings
int32_t st_Buffer_clear_ext(st_Buffer *buffer, bool set_data_to_zero) { return
    st_Buffer_clear(buffer, set_data_to_zero); }
st_buffer_size_t st_Buffer_get_capacity_ext(const st_Buffer *buffer) { return
    st_Buffer_get_capacity(buffer); }
st_buffer_addr_t st_Buffer_get_data_begin_addr_ext(const st_Buffer *buffer) { return
    st_Buffer_get_data_begin_addr(buffer); }
st_buffer_addr_t st_Buffer_get_data_end_addr_ext(const st_Buffer *buffer) { return
    st_Buffer_get_data_end_addr(buffer); }
st_buffer_size_t st_Buffer_get_header_size_ext(const st_Buffer *buffer) { return
    st_Buffer_get_header_size(buffer); }
st_buffer_size_t st_Buffer_get_max_num_of_dataptrs_ext(const st_Buffer *buffer) { return
    st_Buffer_get_max_num_of_dataptrs(buffer); }
st_buffer_size_t st_Buffer_get_max_num_of_garbage_ranges_ext(const st_Buffer *buffer) { return
    st_Buffer_get_max_num_of_garbage_ranges(buffer); }
st_buffer_size_t st_Buffer_get_max_num_of_objects_ext(const st_Buffer *buffer) { return
    st_Buffer_get_max_num_of_objects(buffer); }
st_buffer_size_t st_Buffer_get_max_num_of_slots_ext(const st_Buffer *buffer) { return
    st_Buffer_get_max_num_of_slots(buffer); }
st_buffer_size_t st_Buffer_get_num_of_dataptrs_ext(const st_Buffer *buffer) { return
    st_Buffer_get_num_of_dataptrs(buffer); }
st_buffer_size_t st_Buffer_get_num_of_garbage_ranges_ext(const st_Buffer *buffer) { return
    st_Buffer_get_num_of_garbage_ranges(buffer); }
st_buffer_size_t st_Buffer_get_num_of_objects_ext(const st_Buffer *buffer) { return
    st_Buffer_get_num_of_objects(buffer); }
st_buffer_size_t st_Buffer_get_num_of_slots_ext(const st_Buffer *buffer) { return
    st_Buffer_get_num_of_slots(buffer); }
st_buffer_size_t st_Buffer_get_size_ext(const st_Buffer *buffer) { return
    st_Buffer_get_size(buffer); }
st_buffer_size_t st_Buffer_get_slot_size_ext(const st_Buffer *buffer) { return
    st_Buffer_get_slot_size(buffer); }
bool st_Buffer_needs_remapping_ext(const st_Buffer *buffer) { return
    st_Buffer_needs_remapping(buffer); }
int32_t st_Buffer_refresh_ext(st_Buffer *buffer) { return st_Buffer_refresh(buffer); }
int32_t st_Buffer_remap_ext(st_Buffer *buffer) { return st_Buffer_remap(buffer); }
int32_t st_Buffer_reserve_capacity_ext(st_Buffer *buffer, st_buffer_size_t capacity) { return
    st_Buffer_reserve_capacity(buffer, capacity); }
int32_t st_Buffer_reserve_ext(st_Buffer *buffer, st_buffer_size_t max_num_objects, st_buffer_size_t
    max_num_slots, st_buffer_size_t max_num_dataptrs, st_buffer_size_t max_num_garbage_ranges) {
    return st_Buffer_reserve(buffer, max_num_objects, max_num_slots, max_num_dataptrs,
    max_num_garbage_ranges); }
int32_t st_Buffer_reset_detailed_ext(st_Buffer *buffer, st_buffer_size_t max_num_objects,
    st_buffer_size_t max_num_slots, st_buffer_size_t max_num_dataptrs, st_buffer_size_t
    max_num_garbage_ranges) { return st_Buffer_reset_detailed(buffer, max_num_objects,
    max_num_slots, max_num_dataptrs, max_num_garbage_ranges); }
int32_t st_Buffer_reset_ext(st_Buffer *buffer) { return st_Buffer_reset(buffer); }
int64_t st_ElemByElemConfig_get_particles_store_index_details_ext( const st_ElemByElemConfig
    *config, int64_t particle_id, int64_t at_element, int64_t at_turn) { return
    st_ElemByElemConfig_get_particles_store_index_details(config, particle_id, at_element,
    at_turn); }
int32_t st_ElemByElemConfig_init_detailed_ext(st_ElemByElemConfig *config, int64_t order, int64_t
    min_particle_id, int64_t max_particle_id, int64_t min_element_id, int64_t max_element_id,
    int64_t min_turn, int64_t max_turn, bool is_rolling) { return
    st_ElemByElemConfig_init_detailed(config, order, min_particle_id, max_particle_id,
    min_element_id, max_element_id, min_turn, max_turn, is_rolling); }
st_Particles *st_Particles_add_copy_ext(st_Buffer *buffer, const st_Particles *orig) { return
    st_Particles_add_copy(buffer, orig); }
st_buffer_size_t st_Particles_buffer_get_num_of_particle_blocks_ext(const st_Buffer *buffer) {
    return st_Particles_buffer_get_num_of_particle_blocks(buffer); }
st_Particles *st_Particles_buffer_get_particles_ext(st_Buffer *buffer, st_buffer_size_t index) {
    return st_Particles_buffer_get_particles(buffer, index); }
st_buffer_size_t st_Particles_buffer_get_total_num_of_particles_ext(const st_Buffer *buffer) {
    return st_Particles_buffer_get_total_num_of_particles(buffer); }
void st_Particles_calculate_difference_ext(const st_Particles *lhs, const st_Particles *rhs,
    st_Particles *diff) { st_Particles_calculate_difference(lhs, rhs, diff); }
int32_t st_Particles_copy_ext(st_Particles *dest, const st_Particles *src) { return
    st_Particles_copy(dest, src); }
int64_t st_Particles_get_num_of_particles_ext(const st_Particles *p) { return
    st_Particles_get_num_of_particles(p); }
st_Particles *st_Particles_new_ext(st_Buffer *buffer, st_buffer_size_t num_particles) { return
    st_Particles_new(buffer, num_particles); }

// TrackJobNew names
// The collect flags actually honoured (particles 0x01, beam elements 0x02,
// output 0x04; track/definitions.h) are returned, as the reference does.
uint16_t st_TrackJobNew_collect_detailed(st_TrackJobBaseNew *job, uint16_t flags)
{
    if (!job) return 0;
    st_TrackJob_collect_detailed(job, flags);
    return (uint16_t)(flags & 0x07);
}
st_AssignAddressItem *st_TrackJobNew_add_assign_address_item(st_TrackJobBaseNew *job, const
    st_AssignAddressItem *item) { return st_TrackJob_add_assign_address_item(job, item); }
st_AssignAddressItem *st_TrackJobNew_add_assign_address_item_detailed( st_TrackJobBaseNew *job,
    st_object_type_id_t dest_type_id, st_buffer_size_t dest_buffer_id, st_buffer_size_t
    dest_elem_index, st_buffer_size_t dest_pointer_offset, st_object_type_id_t src_type_id,
    st_buffer_size_t src_buffer_id, st_buffer_size_t src_elem_index, st_buffer_size_t
    src_pointer_offset) { return st_TrackJob_add_assign_address_item_detailed(job, dest_type_id,
    dest_buffer_id, dest_elem_index, dest_pointer_offset, src_type_id, src_buffer_id,
    src_elem_index, src_pointer_offset); }
st_buffer_size_t st_TrackJobNew_add_stored_buffer(st_TrackJobBaseNew *job, st_Buffer *buffer, bool
    take_ownership, bool delete_ptr_after_move) { return st_TrackJob_add_stored_buffer(job, buffer,
    take_ownership, delete_ptr_after_move); }
int32_t st_TrackJobNew_assign_addresses(st_TrackJobBaseNew *job, st_buffer_size_t dest_buffer_id,
    st_buffer_size_t src_buffer_id) { return st_TrackJob_assign_addresses(job, dest_buffer_id,
    src_buffer_id); }
int32_t st_TrackJobNew_assign_all_addresses(st_TrackJobBaseNew *job) { return
    st_TrackJob_assign_all_addresses(job); }
int32_t st_TrackJobNew_collect_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t buffer_id) {
    return st_TrackJob_collect_stored_buffer(job, buffer_id); }
int32_t st_TrackJobNew_commit_address_assignments(st_TrackJobBaseNew *job) { return
    st_TrackJob_commit_address_assignments(job); }
const st_Buffer *st_TrackJobNew_const_stored_buffer(const st_TrackJobBaseNew *job, st_buffer_size_t
    buffer_id) { return st_TrackJob_const_stored_buffer(job, buffer_id); }
st_buffer_size_t st_TrackJobNew_create_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t
    buffer_capacity) { return st_TrackJob_create_stored_buffer(job, buffer_capacity); }
void st_TrackJobNew_disable_collect_beam_elements(st_TrackJobBaseNew *job) {
    st_TrackJob_disable_collect_beam_elements(job); }
void st_TrackJobNew_disable_collect_output(st_TrackJobBaseNew *job) {
    st_TrackJob_disable_collect_output(job); }
void st_TrackJobNew_enable_collect_beam_elements(st_TrackJobBaseNew *job) {
    st_TrackJob_enable_collect_beam_elements(job); }
void st_TrackJobNew_enable_collect_output(st_TrackJobBaseNew *job) {
    st_TrackJob_enable_collect_output(job); }
st_buffer_size_t st_TrackJobNew_get_beam_monitor_index(const st_TrackJobBaseNew *job,
    st_buffer_size_t n) { return st_TrackJob_get_beam_monitor_index(job, n); }
const st_buffer_size_t *st_TrackJobNew_get_beam_monitor_indices_begin(const st_TrackJobBaseNew
    *job) { return st_TrackJob_get_beam_monitor_indices_begin(job); }
const st_buffer_size_t *st_TrackJobNew_get_beam_monitor_indices_end(const st_TrackJobBaseNew *job)
    { return st_TrackJob_get_beam_monitor_indices_end(job); }
bool st_TrackJobNew_get_default_elem_by_elem_config_rolling_flag(const st_TrackJobBaseNew *job) {
    return st_TrackJob_get_default_elem_by_elem_config_rolling_flag(job); }
const st_ElemByElemConfig *st_TrackJobNew_get_elem_by_elem_config(const st_TrackJobBaseNew *job) {
    return st_TrackJob_get_elem_by_elem_config(job); }
int64_t st_TrackJobNew_get_elem_by_elem_config_order(const st_TrackJobBaseNew *job) { return
    st_TrackJob_get_elem_by_elem_config_order(job); }
int64_t st_TrackJobNew_get_max_element_id(const st_TrackJobBaseNew *job) { return
    st_TrackJob_get_max_element_id(job); }
int64_t st_TrackJobNew_get_max_initial_turn_id(const st_TrackJobBaseNew *job) { return
    st_TrackJob_get_max_initial_turn_id(job); }
int64_t st_TrackJobNew_get_max_particle_id(const st_TrackJobBaseNew *job) { return
    st_TrackJob_get_max_particle_id(job); }
int64_t st_TrackJobNew_get_min_element_id(const st_TrackJobBaseNew *job) { return
    st_TrackJob_get_min_element_id(job); }
int64_t st_TrackJobNew_get_min_initial_turn_id(const st_TrackJobBaseNew *job) { return
    st_TrackJob_get_min_initial_turn_id(job); }
int64_t st_TrackJobNew_get_min_particle_id(const st_TrackJobBaseNew *job) { return
    st_TrackJob_get_min_particle_id(job); }
st_buffer_size_t st_TrackJobNew_get_num_elem_by_elem_turns(const st_TrackJobBaseNew *job) { return
    st_TrackJob_get_num_elem_by_elem_turns(job); }
st_buffer_size_t st_TrackJobNew_get_particle_set_index(const st_TrackJobBaseNew *job,
    st_buffer_size_t n) { return st_TrackJob_get_particle_set_index(job, n); }
const st_buffer_size_t *st_TrackJobNew_get_particle_set_indices_begin(const st_TrackJobBaseNew
    *job) { return st_TrackJob_get_particle_set_indices_begin(job); }
const st_buffer_size_t *st_TrackJobNew_get_particle_set_indices_end(const st_TrackJobBaseNew *job)
    { return st_TrackJob_get_particle_set_indices_end(job); }
bool st_TrackJobNew_has_assign_address_item(const st_TrackJobBaseNew *job, const
    st_AssignAddressItem *item) { return st_TrackJob_has_assign_address_item(job, item); }
bool st_TrackJobNew_has_assign_item_by_index(const st_TrackJobBaseNew *job, st_buffer_size_t
    dest_buffer_id, st_buffer_size_t src_buffer_id, st_buffer_size_t assign_item_index) { return
    st_TrackJob_has_assign_item_by_index(job, dest_buffer_id, src_buffer_id, assign_item_index); }
bool st_TrackJobNew_has_assign_items(const st_TrackJobBaseNew *job, st_buffer_size_t
    dest_buffer_id, st_buffer_size_t src_buffer_id) { return st_TrackJob_has_assign_items(job,
    dest_buffer_id, src_buffer_id); }
bool st_TrackJobNew_has_elem_by_elem_config(const st_TrackJobBaseNew *job) { return
    st_TrackJob_has_elem_by_elem_config(job); }
bool st_TrackJobNew_has_stored_buffers(const st_TrackJobBaseNew *job) { return
    st_TrackJob_has_stored_buffers(job); }
st_buffer_size_t st_TrackJobNew_index_of_assign_address_item(const st_TrackJobBaseNew *job, const
    st_AssignAddressItem *item) { return st_TrackJob_index_of_assign_address_item(job, item); }
bool st_TrackJobNew_is_collecting_beam_elements(const st_TrackJobBaseNew *job) { return
    st_TrackJob_is_collecting_beam_elements(job); }
bool st_TrackJobNew_is_collecting_output(const st_TrackJobBaseNew *job) { return
    st_TrackJob_is_collecting_output(job); }
bool st_TrackJobNew_is_elem_by_elem_config_rolling(const st_TrackJobBaseNew *job) { return
    st_TrackJob_is_elem_by_elem_config_rolling(job); }
st_buffer_size_t st_TrackJobNew_max_stored_buffer_id(const st_TrackJobBaseNew *job) { return
    st_TrackJob_max_stored_buffer_id(job); }
st_buffer_size_t st_TrackJobNew_min_stored_buffer_id(const st_TrackJobBaseNew *job) { return
    st_TrackJob_min_stored_buffer_id(job); }
st_buffer_size_t st_TrackJobNew_num_assign_items(const st_TrackJobBaseNew *job, st_buffer_size_t
    dest_buffer_id, st_buffer_size_t src_buffer_id) { return st_TrackJob_num_assign_items(job,
    dest_buffer_id, src_buffer_id); }
st_buffer_size_t st_TrackJobNew_num_stored_buffers(const st_TrackJobBaseNew *job) { return
    st_TrackJob_num_stored_buffers(job); }
bool st_TrackJobNew_owns_stored_buffer(const st_TrackJobBaseNew *job, st_buffer_size_t buffer_id) {
    return st_TrackJob_owns_stored_buffer(job, buffer_id); }
const st_AssignAddressItem *st_TrackJobNew_ptr_assign_address_item( const st_TrackJobBaseNew *job,
    const st_AssignAddressItem *item) { return st_TrackJob_ptr_assign_address_item(job, item); }
const st_AssignAddressItem *st_TrackJobNew_ptr_assign_address_item_by_index( const
    st_TrackJobBaseNew *job, st_buffer_size_t dest_buffer_id, st_buffer_size_t src_buffer_id,
    st_buffer_size_t assign_address_item_index) { return
    st_TrackJob_ptr_assign_address_item_by_index(job, dest_buffer_id, src_buffer_id,
    assign_address_item_index); }
int32_t st_TrackJobNew_push_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t buffer_id) {
    return st_TrackJob_push_stored_buffer(job, buffer_id); }
int32_t st_TrackJobNew_remove_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t buffer_id) {
    return st_TrackJob_remove_stored_buffer(job, buffer_id); }
void st_TrackJobNew_set_default_elem_by_elem_config_rolling_flag(st_TrackJobBaseNew *job, bool
    rolling) { st_TrackJob_set_default_elem_by_elem_config_rolling_flag(job, rolling); }
st_Buffer *st_TrackJobNew_stored_buffer(st_TrackJobBaseNew *job, st_buffer_size_t buffer_id) {
    return st_TrackJob_stored_buffer(job, buffer_id); }
st_buffer_size_t st_TrackJobNew_total_num_assign_items(const st_TrackJobBaseNew *job) { return
    st_TrackJob_total_num_assign_items(job); }

// The legacy TrackJob's names for the particle-address calls (track_job.h:478-492)
int32_t st_TrackJob_fetch_particles_addr(st_TrackJob *job)
{
    return st_TrackJob_fetch_particle_addresses(job);
}
int32_t st_TrackJob_clear_particles_addr(st_TrackJob *job, st_buffer_size_t index)
{
    return st_TrackJob_clear_particle_addresses(job, index);
}
int32_t st_TrackJob_clear_all_particles_addr(st_TrackJob *job)
{
    return st_TrackJob_clear_all_particle_addresses(job);
}
const st_ParticlesAddr *st_TrackJob_particles_addr(const st_TrackJob *job, st_buffer_size_t index)
{
    return st_TrackJob_particle_addresses(job, index);
}

}  // extern "C"

// output_buffer.cpp -- planning and laying out the tracking output buffer on
// the host: which outputs a run needs, how large the buffer must be, the
// Particles blocks themselves and the addresses that point the beam
// monitors and the elem-by-elem configuration at them.
//
// Reference interface: sixtracklib/common/output/output_buffer.h:42-260
// (implementation output_buffer.c:24-516), be_monitor/output_buffer.h:20-135
// (be_monitor/output_buffer.c, be_monitor/output_buffer.h:240-355),
// output/elem_by_elem_output_buffer.h:117-262 (elem_by_elem_output_buffer.c)
// and output/elem_by_elem_config.c:366-375.
//
// Everything works on one "span": the particle-id, element-id and turn
// ranges that the particles and the lattice cover.  The element-id range is
// taken from the lattice the way the reference does: leading objects that
// are not beam elements (particles, lines, configurations) shift the first
// element id, and the last id is the first plus the number of beam
// elements minus one.
#include <algorithm>
#include <climits>
#include <cstdlib>

#include "common.h"

namespace {

constexpr uint32_t kNeedElemByElem = 0x01;  // output_buffer.h:34-36
constexpr uint32_t kNeedMonitors = 0x02;    // output_buffer.h:38-40
constexpr uint64_t kParticleColumns = 21;   // particles/definitions.h:46
constexpr uint64_t kParticlesStructWords = 22;
constexpr uint64_t kTypeLine = 1024;             // objects_type_id.h:43
constexpr uint64_t kTypeInvalid = 0x7fffffff;   // objects_type_id.h:53

struct Span {
    int64_t min_pid = INT64_MAX, max_pid = INT64_MIN;
    int64_t min_elem = INT64_MAX, max_elem = INT64_MIN;
    int64_t min_turn = INT64_MAX, max_turn = INT64_MIN;
};

// Particle ids count by magnitude (a negative id marks a particle that was
// lost in older files); particles.h:2359-2450.
bool widen_by_particles(Span &s, const st_Particles *p)
{
    if (!p || p->num_particles <= 0) return false;
    for (int64_t i = 0; i < p->num_particles; ++i) {
        int64_t const pid = p->particle_id[i] < 0 ? -p->particle_id[i] : p->particle_id[i];
        s.min_pid = std::min(s.min_pid, pid);
        s.max_pid = std::max(s.max_pid, pid);
        s.min_elem = std::min(s.min_elem, p->at_element_id[i]);
        s.max_elem = std::max(s.max_elem, p->at_element_id[i]);
        s.min_turn = std::min(s.min_turn, p->at_turn[i]);
        s.max_turn = std::max(s.max_turn, p->at_turn[i]);
    }
    return true;
}

bool is_beam_element(uint64_t type_id)
{
    return type_id != 0 && type_id != ST_OBJECT_TYPE_PARTICLE && type_id != kTypeInvalid &&
           type_id != kTypeLine && type_id != ST_OBJECT_TYPE_ELEM_BY_ELEM_CONF;
}

// Element-id range of the lattice (elem_by_elem_output_buffer.h:162-262).
bool widen_by_lattice(Span &s, const st_Buffer *eb)
{
    const st_Object *it = st_Buffer_get_const_objects_begin(eb);
    const st_Object *end = st_Buffer_get_const_objects_end(eb);
    if (!it || it == end) return false;
    int64_t first = 0;
    while (it != end && !is_beam_element(it->type_id)) {
        ++first;
        ++it;
    }
    int64_t count = 0;
    for (; it != end; ++it)
        if (is_beam_element(it->type_id)) ++count;
    if (count == 0) return false;
    s.min_elem = std::min(s.min_elem, first);
    s.max_elem = std::max(s.max_elem, first + count - 1);
    return true;
}

bool span_of_particles(const st_Particles *p, const st_Buffer *eb, Span *s)
{
    *s = Span();
    return widen_by_particles(*s, p) && widen_by_lattice(*s, eb);
}

bool span_of_sets(const st_Buffer *pb, uint64_t nsets, const st_buffer_size_t *idx,
                  const st_Buffer *eb, Span *s)
{
    *s = Span();
    if (!pb || !idx || nsets == 0 || st_Buffer_get_num_of_objects(pb) == 0) return false;
    for (uint64_t k = 0; k < nsets; ++k)
        if (!widen_by_particles(*s, st_Particles_buffer_get_const_particles(pb, idx[k])))
            return false;
    return widen_by_lattice(*s, eb);
}

// Slots of one Particles object of n particles with 8-byte slots
// (particles.h:1808-1840): the struct and one column per field.
uint64_t particles_slots(uint64_t n) { return n ? kParticlesStructWords + kParticleColumns * n : 0; }

uint64_t ebe_stored_particles(int64_t min_pid, int64_t max_pid, int64_t min_elem, int64_t max_elem,
                              int64_t min_turn, int64_t max_turn)
{
    if (min_pid < 0 || max_pid < min_pid || min_elem < 0 || max_elem < min_elem || min_turn < 0 ||
        max_turn < min_turn)
        return 0;
    return (uint64_t)(max_pid - min_pid + 1) * (uint64_t)(max_elem - min_elem + 1) *
           (uint64_t)(max_turn - min_turn + 1);
}

st_BeamMonitor *monitor_of(const st_Object &o)
{
    return (o.type_id == ST_OBJECT_TYPE_BEAM_MONITOR && o.begin_addr != 0)
               ? (st_BeamMonitor *)(uintptr_t)o.begin_addr
               : nullptr;
}

struct Sizes {
    uint64_t objects = 0, slots = 0, dataptrs = 0, garbage = 0;
    void add_particles(uint64_t n)
    {
        ++objects;
        dataptrs += kParticleColumns;
        slots += particles_slots(n);
    }
};

// Elem-by-elem share of the output size (elem_by_elem_output_buffer.c:88-172).
bool ebe_sizes(const Span &s, uint64_t until_ebe, Sizes *z)
{
    bool const valid = s.min_pid <= s.max_pid && s.min_turn <= s.max_turn && s.min_pid >= 0 &&
                       s.min_turn >= 0;
    if (!valid) return false;
    if (until_ebe <= (uint64_t)s.min_turn) return true;
    uint64_t const n = ebe_stored_particles(s.min_pid, s.max_pid, s.min_elem, s.max_elem,
                                            s.min_turn, (int64_t)until_ebe - 1);
    if (n == 0) return false;
    z->add_particles(n);
    return true;
}

// Beam-monitor share (be_monitor/output_buffer.c:84-190).  A monitor that
// starts at or after the first turn, or a rolling one, needs all its stores;
// one that started earlier needs the stores it has left.
bool monitor_sizes(const st_Buffer *eb, const Span &s, Sizes *z)
{
    if (s.min_turn < 0 || s.min_pid < 0 || s.min_pid > s.max_pid) return false;
    uint64_t const per_turn = (uint64_t)(s.max_pid - s.min_pid + 1);
    int64_t const first = s.min_turn;
    for (const st_Object *o = st_Buffer_get_const_objects_begin(eb);
         o != st_Buffer_get_const_objects_end(eb); ++o) {
        const st_BeamMonitor *m = monitor_of(*o);
        if (!m) continue;
        uint64_t need = 0;
        if (m->start >= first || m->is_rolling != 0) {
            need = per_turn * (uint64_t)m->num_stores;
        } else if (m->skip >= 1) {
            int64_t const already = 1 + (first - m->start) / m->skip;
            if (m->num_stores > already) need = per_turn * (uint64_t)(m->num_stores - already);
        }
        if (need > 0) z->add_particles(need);
    }
    return true;
}

bool buffer_ready(const st_Buffer *b) { return b && !st_Buffer_needs_remapping(b); }

// Appends the elem-by-elem block (elem_by_elem_output_buffer.c:247-351).
bool add_ebe_block(st_Buffer *out, const Span &s, int64_t max_ebe_turn, uint64_t *offset)
{
    if (!buffer_ready(out) || s.min_pid < 0 || s.min_pid > s.max_pid || s.min_elem < 0 ||
        s.min_elem > s.max_elem || s.min_turn < 0 || s.min_turn > max_ebe_turn)
        return false;
    uint64_t const first = st_Buffer_get_num_of_objects(out);
    uint64_t const n =
        ebe_stored_particles(s.min_pid, s.max_pid, s.min_elem, s.max_elem, s.min_turn, max_ebe_turn);
    if (n == 0) return false;
    if (!st_Particles_new(out, n)) return false;
    *offset = first;
    return true;
}

// Appends one block per monitor that starts at or after the first turn and
// stores something, and gives the monitor the particle-id range
// (be_monitor/output_buffer.c:247-350).
bool add_monitor_blocks(st_Buffer *eb, st_Buffer *out, const Span &s, uint64_t *offset)
{
    if (s.min_turn < 0 || s.min_pid < 0 || s.max_pid < s.min_pid) return false;
    uint64_t const first = st_Buffer_get_num_of_objects(out);
    uint64_t const per_turn = (uint64_t)(s.max_pid - s.min_pid + 1);
    uint64_t const ne = st_Buffer_get_num_of_objects(eb);
    for (uint64_t i = 0; i < ne; ++i) {
        // eb and out are distinct buffers: appending to out leaves eb in place
        st_BeamMonitor *m = monitor_of(*st_Buffer_get_const_object(eb, i));
        if (!m || m->start < s.min_turn || m->num_stores <= 0) continue;
        if (!st_Particles_new(out, per_turn * (uint64_t)m->num_stores)) return false;
        m->min_particle_id = s.min_pid;
        m->max_particle_id = s.max_pid;
        m->out_address = 0;
    }
    *offset = first;
    return true;
}

}  // namespace

extern "C" {

bool st_OutputBuffer_requires_output_buffer_ext(uint32_t flags) { return flags != 0; }
bool st_OutputBuffer_requires_elem_by_elem_output_ext(uint32_t flags)
{
    return (flags & kNeedElemByElem) != 0;
}
bool st_OutputBuffer_requires_beam_monitor_output_ext(uint32_t flags)
{
    return (flags & kNeedMonitors) != 0;
}

uint32_t st_OutputBuffer_required_for_tracking_detailed(
    const st_Buffer *eb, int64_t min_pid, int64_t max_pid, int64_t min_elem, int64_t max_elem,
    int64_t min_turn, int64_t max_turn, st_buffer_size_t until_ebe)
{
    uint32_t flags = 0;
    if (min_pid < 0 || min_pid > max_pid || min_elem < 0 || min_elem > max_elem ||
        min_turn < 0 || min_turn > max_turn)
        return flags;
    uint64_t const ne = st_Buffer_get_num_of_objects(eb);
    if (until_ebe > (uint64_t)min_turn && ne > 0) flags |= kNeedElemByElem;
    for (const st_Object *o = st_Buffer_get_const_objects_begin(eb);
         ne > 0 && o != st_Buffer_get_const_objects_end(eb); ++o) {
        const st_BeamMonitor *m = monitor_of(*o);
        if (m && o->size >= sizeof(st_BeamMonitor) && m->num_stores > 0) {
            flags |= kNeedMonitors;
            break;
        }
    }
    return flags;
}

uint32_t st_OutputBuffer_required_for_tracking(const st_Particles *p, const st_Buffer *eb,
                                               st_buffer_size_t until_ebe)
{
    Span s;
    if (!span_of_particles(p, eb, &s)) return 0;
    return st_OutputBuffer_required_for_tracking_detailed(eb, s.min_pid, s.max_pid, s.min_elem,
                                                          s.max_elem, s.min_turn, s.max_turn,
                                                          until_ebe);
}

uint32_t st_OutputBuffer_required_for_tracking_of_particle_sets(const st_Buffer *pb,
                                                                st_buffer_size_t nsets,
                                                                const st_buffer_size_t *idx,
                                                                const st_Buffer *eb,
                                                                st_buffer_size_t until_ebe)
{
    Span s;
    if (!span_of_sets(pb, nsets, idx, eb, &s)) return 0;
    return st_OutputBuffer_required_for_tracking_detailed(eb, s.min_pid, s.max_pid, s.min_elem,
                                                          s.max_elem, s.min_turn, s.max_turn,
                                                          until_ebe);
}

int32_t st_OutputBuffer_calculate_output_buffer_params_detailed(
    const st_Buffer *eb, int64_t min_pid, int64_t max_pid, int64_t min_elem, int64_t max_elem,
    int64_t min_turn, int64_t max_turn, st_buffer_size_t until_ebe, st_buffer_size_t *num_objects,
    st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs, st_buffer_size_t *num_garbage,
    st_buffer_size_t slot_size)
{
    if (!eb || slot_size != 8) {
        stg::set_error("OutputBuffer_calculate_output_buffer_params: needs a beam-elements "
                       "buffer and 8-byte slots");
        return -1;
    }
    Span s;
    s.min_pid = min_pid;
    s.max_pid = max_pid;
    s.min_elem = min_elem;
    s.max_elem = max_elem;
    s.min_turn = min_turn;
    s.max_turn = max_turn;
    Sizes z;
    if ((until_ebe > 0 && !ebe_sizes(s, until_ebe, &z)) || !monitor_sizes(eb, s, &z)) return -1;
    if (num_objects) *num_objects = z.objects;
    if (num_slots) *num_slots = z.slots;
    if (num_dataptrs) *num_dataptrs = z.dataptrs;
    if (num_garbage) *num_garbage = z.garbage;
    return 0;
}

int32_t st_OutputBuffer_calculate_output_buffer_params(
    const st_Buffer *eb, const st_Particles *p, st_buffer_size_t until_ebe,
    st_buffer_size_t *num_objects, st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs,
    st_buffer_size_t *num_garbage, st_buffer_size_t slot_size)
{
    Span s;
    if (!span_of_particles(p, eb, &s)) return -1;
    return st_OutputBuffer_calculate_output_buffer_params_detailed(
        eb, s.min_pid, s.max_pid, s.min_elem, s.max_elem, s.min_turn, s.max_turn, until_ebe,
        num_objects, num_slots, num_dataptrs, num_garbage, slot_size);
}

int32_t st_OutputBuffer_calculate_output_buffer_params_for_particles_sets(
    const st_Buffer *eb, const st_Buffer *pb, st_buffer_size_t nsets,
    const st_buffer_size_t *idx, st_buffer_size_t until_ebe, st_buffer_size_t *num_objects,
    st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs, st_buffer_size_t *num_garbage,
    st_buffer_size_t slot_size)
{
    Span s;
    if (!span_of_sets(pb, nsets, idx, eb, &s)) return -1;
    return st_OutputBuffer_calculate_output_buffer_params_detailed(
        eb, s.min_pid, s.max_pid, s.min_elem, s.max_elem, s.min_turn, s.max_turn, until_ebe,
        num_objects, num_slots, num_dataptrs, num_garbage, slot_size);
}

int32_t st_OutputBuffer_prepare_detailed(st_Buffer *eb, st_Buffer *out, int64_t min_pid,
                                         int64_t max_pid, int64_t min_elem, int64_t max_elem,
                                         int64_t min_turn, int64_t max_turn,
                                         st_buffer_size_t until_ebe,
                                         st_buffer_size_t *ebe_offset,
                                         st_buffer_size_t *monitor_offset,
                                         int64_t *max_ebe_turn)
{
    (void)max_turn;
    if (!buffer_ready(eb) || !buffer_ready(out)) {
        stg::set_error("OutputBuffer_prepare: missing beam-elements or output buffer");
        return -1;
    }
    Span s;
    s.min_pid = min_pid;
    s.max_pid = max_pid;
    s.min_elem = min_elem;
    s.max_elem = max_elem;
    s.min_turn = min_turn;
    uint64_t ebe_off = 0, mon_off = 0;
    int64_t ebe_turn = 0;
    if (min_turn >= 0 && until_ebe > (uint64_t)min_turn) {
        ebe_turn = (int64_t)until_ebe - 1;
        if (!add_ebe_block(out, s, ebe_turn, &ebe_off)) return -1;
    }
    if (!add_monitor_blocks(eb, out, s, &mon_off)) return -1;
    if (ebe_offset) *ebe_offset = ebe_off;
    if (monitor_offset) *monitor_offset = mon_off;
    if (max_ebe_turn) *max_ebe_turn = ebe_turn;
    return 0;
}

int32_t st_OutputBuffer_prepare(st_Buffer *eb, st_Buffer *out, const st_Particles *p,
                                st_buffer_size_t until_ebe, st_buffer_size_t *ebe_offset,
                                st_buffer_size_t *monitor_offset, int64_t *min_turn)
{
    Span s;
    if (!span_of_particles(p, eb, &s)) return -1;
    int32_t const r = st_OutputBuffer_prepare_detailed(eb, out, s.min_pid, s.max_pid, s.min_elem,
                                                       s.max_elem, s.min_turn, s.max_turn,
                                                       until_ebe, ebe_offset, monitor_offset,
                                                       nullptr);
    if (r == 0 && min_turn) *min_turn = s.min_turn;
    return r;
}

int32_t st_OutputBuffer_prepare_for_particle_sets(st_Buffer *eb, st_Buffer *out,
                                                  const st_Buffer *pb, st_buffer_size_t nsets,
                                                  const st_buffer_size_t *idx,
                                                  st_buffer_size_t until_ebe,
                                                  st_buffer_size_t *ebe_offset,
                                                  st_buffer_size_t *monitor_offset,
                                                  int64_t *min_turn)
{
    Span s;
    if (!span_of_sets(pb, nsets, idx, eb, &s)) return -1;
    int32_t const r = st_OutputBuffer_prepare_detailed(eb, out, s.min_pid, s.max_pid, s.min_elem,
                                                       s.max_elem, s.min_turn, s.max_turn,
                                                       until_ebe, ebe_offset, monitor_offset,
                                                       nullptr);
    if (r == 0 && min_turn) *min_turn = s.min_turn;
    return r;
}

// ------------------------------------------------------------ monitors
int32_t st_BeamMonitor_calculate_output_buffer_params_detailed(
    const st_Buffer *eb, int64_t min_pid, int64_t max_pid, int64_t min_turn,
    st_buffer_size_t *num_objects, st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs,
    st_buffer_size_t *num_garbage, st_buffer_size_t slot_size)
{
    if (!eb || slot_size != 8) return -1;
    Span s;
    s.min_pid = min_pid;
    s.max_pid = max_pid;
    s.min_turn = min_turn;
    Sizes z;
    if (!monitor_sizes(eb, s, &z)) return -1;
    if (num_objects) *num_objects = z.objects;
    if (num_slots) *num_slots = z.slots;
    if (num_dataptrs) *num_dataptrs = z.dataptrs;
    if (num_garbage) *num_garbage = z.garbage;
    return 0;
}

// The particle-id and turn ranges here start from 0 rather than from the
// first particle (be_monitor/output_buffer.c:33-38): the range always
// includes id 0 and turn 0, so every monitor counts from turn 0.
int32_t st_BeamMonitor_calculate_output_buffer_params(
    const st_Buffer *eb, const st_Particles *p, st_buffer_size_t *num_objects,
    st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs, st_buffer_size_t *num_garbage,
    st_buffer_size_t slot_size)
{
    Span s;
    s.min_pid = s.max_pid = s.min_turn = s.max_turn = 0;
    if (!widen_by_particles(s, p)) return -1;
    return st_BeamMonitor_calculate_output_buffer_params_detailed(
        eb, s.min_pid, s.max_pid, s.min_turn, num_objects, num_slots, num_dataptrs, num_garbage,
        slot_size);
}

int32_t st_BeamMonitor_prepare_output_buffer_detailed(st_Buffer *eb, st_Buffer *out,
                                                      int64_t min_pid, int64_t max_pid,
                                                      int64_t min_turn,
                                                      st_buffer_size_t *offset)
{
    if (!buffer_ready(eb) || !buffer_ready(out)) return -1;
    Span s;
    s.min_pid = min_pid;
    s.max_pid = max_pid;
    s.min_turn = min_turn;
    uint64_t off = 0;
    if (!add_monitor_blocks(eb, out, s, &off)) return -1;
    if (offset) *offset = off;
    return 0;
}

// Ranges from the particles alone (be_monitor/output_buffer.c:192-216).
int32_t st_BeamMonitor_prepare_output_buffer(st_Buffer *eb, st_Buffer *out,
                                             const st_Particles *p, st_buffer_size_t *offset)
{
    Span s;
    if (!widen_by_particles(s, p)) return -1;
    return st_BeamMonitor_prepare_output_buffer_detailed(eb, out, s.min_pid, s.max_pid,
                                                         s.min_turn, offset);
}

// Points each storing monitor at the next Particles block of `out`, from
// object `offset` on (be_monitor/output_buffer.h:240-355).  A block too small
// for the monitor's particle-id range times its stores, or running out of
// blocks while monitors remain, is an error.
int32_t st_BeamMonitor_assign_output_buffer_from_offset(st_Buffer *eb, st_Buffer *out,
                                                        int64_t min_turn,
                                                        st_buffer_size_t offset)
{
    if (!buffer_ready(eb) || !buffer_ready(out)) return -1;
    uint64_t const nout = st_Buffer_get_num_of_objects(out);
    if (offset > nout) return -1;
    uint64_t next = offset;
    uint64_t const ne = st_Buffer_get_num_of_objects(eb);
    for (uint64_t i = 0; i < ne; ++i) {
        st_BeamMonitor *m = monitor_of(*st_Buffer_get_const_object(eb, i));
        if (!m) continue;
        if (m->num_stores > 0 && m->start >= min_turn && next != nout) {
            const st_Particles *blk = st_Particles_buffer_get_const_particles(out, next);
            uint64_t const stored = blk ? (uint64_t)blk->num_particles : 0;
            uint64_t const per_turn = m->max_particle_id >= m->min_particle_id
                                          ? (uint64_t)(m->max_particle_id - m->min_particle_id + 1)
                                          : 0;
            if (per_turn == 0) continue;
            if (!blk || per_turn * (uint64_t)m->num_stores > stored) {
                stg::set_error("BeamMonitor_assign_output_buffer: output block " +
                               std::to_string(next) + " is too small for monitor " +
                               std::to_string(i));
                return -1;
            }
            m->out_address = st_Buffer_get_const_object(out, next)->begin_addr;
            ++next;
        } else if (next == nout) {
            stg::set_error("BeamMonitor_assign_output_buffer: no output block left for element " +
                           std::to_string(i));
            return -1;
        }
    }
    return 0;
}

// The monitors' blocks follow the elem-by-elem block when that one is made
// (be_monitor/output_buffer.c:353-384).
int32_t st_BeamMonitor_assign_output_buffer(st_Buffer *eb, st_Buffer *out, int64_t min_turn,
                                            st_buffer_size_t until_ebe)
{
    if (min_turn < 0) return -1;
    if (until_ebe > (uint64_t)min_turn && st_Buffer_get_num_of_objects(eb) > 1)
        return st_BeamMonitor_assign_output_buffer_from_offset(eb, out, min_turn, 1);
    if (until_ebe == 0 || until_ebe <= (uint64_t)min_turn)
        return st_BeamMonitor_assign_output_buffer_from_offset(eb, out, min_turn, 0);
    return -1;
}

// Every monitor of the lattice gets the particle-id range of `p` and loses
// its output address (be_monitor/output_buffer.c:418-425,
// be_monitor/output_buffer.h:200-238).  The range is that of the particle
// ids as stored; the reference seeds its scan with at_element_id[0]
// (particles.h:5958-5961), which only differs when particle 0's element id
// lies outside the particle-id range.
int32_t st_BeamMonitor_setup_for_particles_all(st_Buffer *eb, const st_Particles *p)
{
    if (!buffer_ready(eb) || !p || p->num_particles <= 0) return -1;
    int64_t lo = p->particle_id[0], hi = p->particle_id[0];
    for (int64_t i = 1; i < p->num_particles; ++i) {
        lo = std::min(lo, p->particle_id[i]);
        hi = std::max(hi, p->particle_id[i]);
    }
    for (st_Object *o = st_Buffer_get_objects_begin(eb); o != st_Buffer_get_objects_end(eb); ++o) {
        st_BeamMonitor *m = monitor_of(*o);
        if (!m) continue;
        m->min_particle_id = lo;
        m->max_particle_id = hi;
        m->out_address = 0;
    }
    return 0;
}

// ------------------------------------------------------ elem-by-elem
int32_t st_ElemByElemConfig_calculate_output_buffer_params_detailed(
    int64_t min_pid, int64_t max_pid, int64_t min_elem, int64_t max_elem, int64_t min_turn,
    int64_t max_turn, st_buffer_size_t until_ebe, st_buffer_size_t *num_objects,
    st_buffer_size_t *num_slots, st_buffer_size_t *num_dataptrs, st_buffer_size_t *num_garbage,
    st_buffer_size_t slot_size)
{
    if (slot_size != 8) return -1;
    Span s;
    s.min_pid = min_pid;
    s.max_pid = max_pid;
    s.min_elem = min_elem;
    s.max_elem = max_elem;
    s.min_turn = min_turn;
    s.max_turn = max_turn;
    Sizes z;
    if (!ebe_sizes(s, until_ebe, &z)) return -1;
    if (num_objects) *num_objects = z.objects;
    if (num_slots) *num_slots = z.slots;
    if (num_dataptrs) *num_dataptrs = z.dataptrs;
    if (num_garbage) *num_garbage = z.garbage;
    return 0;
}

int32_t st_ElemByElemConfig_prepare_output_buffer_detailed(st_Buffer *out, int64_t min_pid,
                                                           int64_t max_pid, int64_t min_elem,
                                                           int64_t max_elem, int64_t min_turn,
                                                           int64_t max_ebe_turn,
                                                           st_buffer_size_t *offset)
{
    Span s;
    s.min_pid = min_pid;
    s.max_pid = max_pid;
    s.min_elem = min_elem;
    s.max_elem = max_elem;
    s.min_turn = min_turn;
    uint64_t off = 0;
    if (!add_ebe_block(out, s, max_ebe_turn, &off)) return -1;
    if (offset) *offset = off;
    return 0;
}

// The configuration's store address becomes the Particles block at object
// `offset` of `out` (output_buffer.h:314-353, elem_by_elem_config.c:366-375).
int32_t st_ElemByElemConfig_assign_output_buffer(st_ElemByElemConfig *c, st_Buffer *out,
                                                 st_buffer_size_t offset)
{
    if (!c || !buffer_ready(out)) return -1;
    const st_Particles *blk = st_Particles_buffer_get_const_particles(out, offset);
    if (!blk) return -1;
    c->out_store_addr = (st_buffer_addr_t)(uintptr_t)blk;
    return 0;
}

// The configuration's field accessors and lifecycle (the reference's
// out-of-line "_ext" copies of elem_by_elem_config.h:532-1160, create and
// delete of elem_by_elem_config.c).  clear empties the ranges (ids -1,
// counts 0, no store address); preset also makes the order invalid (-1)
// and the store rolling.
void st_ElemByElemConfig_clear_ext(st_ElemByElemConfig *c)
{
    if (!c) return;
    c->num_particles_to_store = c->num_elements_to_store = c->num_turns_to_store = 0;
    c->min_particle_id = c->max_particle_id = -1;
    c->min_element_id = c->max_element_id = -1;
    c->min_turn = c->max_turn = -1;
    c->out_store_addr = 0;
}
st_ElemByElemConfig *st_ElemByElemConfig_preset_ext(st_ElemByElemConfig *c)
{
    if (!c) return c;
    st_ElemByElemConfig_clear_ext(c);
    c->order = -1;
    c->is_rolling = 1;
    return c;
}
st_ElemByElemConfig *st_ElemByElemConfig_create(void)
{
    return st_ElemByElemConfig_preset_ext(
        static_cast<st_ElemByElemConfig *>(std::malloc(sizeof(st_ElemByElemConfig))));
}
void st_ElemByElemConfig_delete(st_ElemByElemConfig *c) { std::free(c); }
bool st_ElemByElemConfig_is_active_ext(const st_ElemByElemConfig *c)
{
    return c && c->num_particles_to_store > 0 && c->num_elements_to_store > 0 &&
           c->num_turns_to_store > 0 && c->order != -1;
}
int32_t st_ElemByElemConfig_get_order_ext(const st_ElemByElemConfig *c)
{
    return c ? (int32_t)c->order : -1;  // the reference returns its order enum
}
int64_t st_ElemByElemConfig_get_num_particles_to_store_ext(const st_ElemByElemConfig *c)
{
    return c ? c->num_particles_to_store : 0;
}
int64_t st_ElemByElemConfig_get_num_elements_to_store_ext(const st_ElemByElemConfig *c)
{
    return c ? c->num_elements_to_store : 0;
}
int64_t st_ElemByElemConfig_get_num_turns_to_store_ext(const st_ElemByElemConfig *c)
{
    return c ? c->num_turns_to_store : 0;
}
int64_t st_ElemByElemConfig_get_out_store_num_particles_ext(const st_ElemByElemConfig *c)
{
    return c ? c->num_particles_to_store * c->num_elements_to_store * c->num_turns_to_store : 0;
}
int64_t st_ElemByElemConfig_get_min_particle_id_ext(const st_ElemByElemConfig *c)
{
    return c ? c->min_particle_id : -1;
}
int64_t st_ElemByElemConfig_get_max_particle_id_ext(const st_ElemByElemConfig *c)
{
    return c ? c->max_particle_id : -1;
}
int64_t st_ElemByElemConfig_get_min_element_id_ext(const st_ElemByElemConfig *c)
{
    return c ? c->min_element_id : -1;
}
int64_t st_ElemByElemConfig_get_max_element_id_ext(const st_ElemByElemConfig *c)
{
    return c ? c->max_element_id : -1;
}
int64_t st_ElemByElemConfig_get_min_turn_ext(const st_ElemByElemConfig *c) { return c ? c->min_turn : -1; }
int64_t st_ElemByElemConfig_get_max_turn_ext(const st_ElemByElemConfig *c) { return c ? c->max_turn : -1; }
bool st_ElemByElemConfig_is_rolling_ext(const st_ElemByElemConfig *c) { return c && c->is_rolling != 0; }
st_buffer_addr_t st_ElemByElemConfig_get_output_store_address_ext(const st_ElemByElemConfig *c)
{
    return c ? c->out_store_addr : 0;
}
void st_ElemByElemConfig_set_order_ext(st_ElemByElemConfig *c, int64_t order)
{
    if (c) c->order = order;
}
void st_ElemByElemConfig_set_is_rolling_ext(st_ElemByElemConfig *c, bool is_rolling)
{
    if (c) c->is_rolling = is_rolling ? 1 : 0;
}
void st_ElemByElemConfig_set_output_store_address_ext(st_ElemByElemConfig *c,
                                                      st_buffer_addr_t addr)
{
    if (c) c->out_store_addr = addr;
}

// ------------------------------------------------------------ particles
st_buffer_size_t st_Particles_buffer_get_total_num_of_particles(const st_Buffer *b)
{
    st_buffer_size_t n = 0;
    for (const st_Object *o = st_Buffer_get_const_objects_begin(b);
         o != st_Buffer_get_const_objects_end(b); ++o)
        if (o->type_id == ST_OBJECT_TYPE_PARTICLE)
            n += (st_buffer_size_t)((const st_Particles *)(uintptr_t)o->begin_addr)->num_particles;
    return n;
}

// diff = lhs - rhs, column by column, when all three hold the same number
// of particles (particles.h:3121-3230).
void st_Particles_calculate_difference(const st_Particles *lhs, const st_Particles *rhs,
                                       st_Particles *diff)
{
    if (!lhs || !rhs || !diff || lhs->num_particles <= 0 ||
        rhs->num_particles != lhs->num_particles || diff->num_particles != lhs->num_particles)
        return;
    int64_t const n = lhs->num_particles;
    double *const *lr = &lhs->q0;
    double *const *rr = &rhs->q0;
    double *const *dr = &diff->q0;
    for (int c = 0; c < 17; ++c)
        for (int64_t i = 0; i < n; ++i) dr[c][i] = lr[c][i] - rr[c][i];
    int64_t *const *li = &lhs->particle_id;
    int64_t *const *ri = &rhs->particle_id;
    int64_t *const *di = &diff->particle_id;
    for (int c = 0; c < 4; ++c)
        for (int64_t i = 0; i < n; ++i) di[c][i] = li[c][i] - ri[c][i];
}

}  // extern "C"

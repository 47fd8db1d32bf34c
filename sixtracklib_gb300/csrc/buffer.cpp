// buffer.cpp -- CObjects buffers (NS(Buffer)) on the host.
//
// Image layout (sixtracklib/common/buffer/managed_buffer_minimal.h:396-770,
// buffer/managed_buffer_remap.h:180-644): an 8-word header
//   [base_addr, size_bytes, header_bytes, slots_addr, objects_addr,
//    dataptrs_addr, garbage_addr, 0]
// followed by four sections, each [section_bytes, num_entities, entries...].
// The image always lives at its own base address ("remapped"), so element
// pointers handed out by the *_add functions are directly usable, exactly as
// in the reference.  Growth re-lays the sections out with doubled capacity
// and shifts every stored address; pointers returned earlier become invalid,
// as they do in the reference.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <new>

#include "common.h"

namespace stg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

bool ImageView::open(const void *image, uint64_t max_bytes, std::string *err)
{
    img = static_cast<const uint64_t *>(image);
    auto fail = [&](const char *m) {
        if (err) *err = m;
        return false;
    };
    if (!img || max_bytes < 64) return fail("CObjects image: null or too small");
    base = img[0];
    uint64_t const size = img[1];
    if (size % 8 != 0 || size < 64 || size > max_bytes)
        return fail("CObjects image: inconsistent buffer size");
    size_words = size / 8;
    uint64_t const ow = word_of(img[4]);
    uint64_t const dw = word_of(img[5]);
    if (ow == UINT64_MAX || dw == UINT64_MAX || ow + 2 > size_words || dw + 2 > size_words)
        return fail("CObjects image: section address outside the buffer");
    num_objects = img[ow + 1];
    objs = img + ow + 2;
    if (ow + 2 + 3 * num_objects > size_words)
        return fail("CObjects image: object table overflows the buffer");
    num_dataptrs = img[dw + 1];
    dptrs = img + dw + 2;
    if (dw + 2 + num_dataptrs > size_words)
        return fail("CObjects image: dataptr table overflows the buffer");
    for (uint64_t i = 0; i < num_objects; ++i) {
        uint64_t b = word_of(objs[3 * i]);
        uint64_t n = objs[3 * i + 2];
        if (b == UINT64_MAX || n % 8 != 0 || b + n / 8 > size_words)
            return fail("CObjects image: object outside the buffer");
    }
    return true;
}

}  // namespace stg

using stg::set_error;

// ------------------------------------------------------------ st_Buffer
struct st_Buffer {
    uint64_t *mem = nullptr;
    uint64_t cap_words = 0;
    // section geometry (word offsets of the section headers, capacities)
    uint64_t slots_w = 8, slots_cap = 0;
    uint64_t objs_w = 0, objs_cap = 0;
    uint64_t dptr_w = 0, dptr_cap = 0;
    uint64_t garb_w = 0;
    uint64_t generation = 0;  // bumped on every change (device caches key on it)
};

namespace {

uint64_t *alloc_words(uint64_t n)
{
    void *p = nullptr;
    if (posix_memalign(&p, 64, (size_t)(n * 8)) != 0) return nullptr;
    std::memset(p, 0, (size_t)(n * 8));
    return static_cast<uint64_t *>(p);
}

uint64_t base_of(const st_Buffer *b) { return (uint64_t)(uintptr_t)b->mem; }

uint64_t nslots(const st_Buffer *b) { return b->mem[b->slots_w + 1]; }
uint64_t nobjs(const st_Buffer *b) { return b->mem[b->objs_w + 1]; }
uint64_t ndptrs(const st_Buffer *b) { return b->mem[b->dptr_w + 1]; }

// Write a canonical layout with the given capacities, copying the logical
// content (objects, their words, dataptrs) from `src` (may be null).
bool relayout(st_Buffer *b, const stg::ImageView *src, uint64_t slots_cap,
              uint64_t objs_cap, uint64_t dptr_cap)
{
    uint64_t const slots_w = 8;
    uint64_t const objs_w = slots_w + 2 + slots_cap;
    uint64_t const dptr_w = objs_w + 2 + 3 * objs_cap;
    uint64_t const garb_w = dptr_w + 2 + dptr_cap;
    uint64_t const total = garb_w + 2;
    uint64_t *mem = alloc_words(total);
    if (!mem) {
        set_error("out of host memory for CObjects buffer");
        return false;
    }
    uint64_t const base = (uint64_t)(uintptr_t)mem;
    mem[0] = base;
    mem[1] = total * 8;
    mem[2] = 64;
    mem[3] = base + slots_w * 8;
    mem[4] = base + objs_w * 8;
    mem[5] = base + dptr_w * 8;
    mem[6] = base + garb_w * 8;
    mem[slots_w] = (objs_w - slots_w) * 8;
    mem[objs_w] = (dptr_w - objs_w) * 8;
    mem[dptr_w] = (garb_w - dptr_w) * 8;
    mem[garb_w] = 16;
    uint64_t pos = slots_w + 2;
    uint64_t nd = 0;
    if (src) {
        // objects are copied in order; a word of the old image maps to the
        // new image by (old_word - old_obj_begin) + new_obj_begin
        std::vector<uint64_t> new_begin(src->num_objects);
        std::vector<uint64_t> old_begin(src->num_objects), old_n(src->num_objects);
        for (uint64_t i = 0; i < src->num_objects; ++i) {
            old_begin[i] = src->begin_word(i);
            old_n[i] = src->size_bytes(i) / 8;
            new_begin[i] = pos;
            std::memcpy(mem + pos, src->img + old_begin[i], old_n[i] * 8);
            uint64_t const e = objs_w + 2 + 3 * i;
            mem[e] = base + pos * 8;
            mem[e + 1] = src->type_of(i);
            mem[e + 2] = old_n[i] * 8;
            pos += old_n[i];
        }
        auto map_word = [&](uint64_t w) -> uint64_t {
            for (uint64_t i = 0; i < src->num_objects; ++i)
                if (w >= old_begin[i] && w < old_begin[i] + old_n[i])
                    return new_begin[i] + (w - old_begin[i]);
            return UINT64_MAX;
        };
        // objects are sorted by position in practice: use a moving cursor
        uint64_t cur = 0;
        for (uint64_t k = 0; k < src->num_dataptrs; ++k) {
            uint64_t const fw = src->word_of(src->dptrs[k]);
            if (fw == UINT64_MAX) continue;
            uint64_t nfw = UINT64_MAX;
            if (cur < src->num_objects && fw >= old_begin[cur] &&
                fw < old_begin[cur] + old_n[cur]) {
                nfw = new_begin[cur] + (fw - old_begin[cur]);
            } else {
                for (uint64_t i = 0; i < src->num_objects; ++i)
                    if (fw >= old_begin[i] && fw < old_begin[i] + old_n[i]) {
                        cur = i;
                        nfw = new_begin[i] + (fw - old_begin[i]);
                        break;
                    }
            }
            if (nfw == UINT64_MAX) continue;
            uint64_t const tw = src->word_of(src->img[fw]);
            uint64_t const ntw = (tw == UINT64_MAX) ? UINT64_MAX : map_word(tw);
            if (ntw != UINT64_MAX) mem[nfw] = base + ntw * 8;
            mem[dptr_w + 2 + nd] = base + nfw * 8;
            ++nd;
        }
        // interpolated space charge: field 6 is a plain address (not a
        // dataptr); when it names an object of this buffer, move it along
        for (uint64_t i = 0; i < src->num_objects; ++i) {
            if (src->type_of(i) != ST_OBJECT_TYPE_SC_INTERPOLATED_PROF || old_n[i] < 7) continue;
            uint64_t const tw = src->word_of(src->img[old_begin[i] + 6]);
            for (uint64_t t = 0; t < src->num_objects && tw != UINT64_MAX; ++t)
                if (old_begin[t] == tw) {
                    mem[new_begin[i] + 6] = base + new_begin[t] * 8;
                    break;
                }
        }
        mem[objs_w + 1] = src->num_objects;
    } else {
        mem[objs_w + 1] = 0;
    }
    mem[slots_w + 1] = pos - (slots_w + 2);
    mem[dptr_w + 1] = nd;
    mem[garb_w + 1] = 0;
    std::free(b->mem);
    b->mem = mem;
    b->cap_words = total;
    b->slots_w = slots_w;
    b->slots_cap = slots_cap;
    b->objs_w = objs_w;
    b->objs_cap = objs_cap;
    b->dptr_w = dptr_w;
    b->dptr_cap = dptr_cap;
    b->garb_w = garb_w;
    ++b->generation;
    return true;
}

bool ensure(st_Buffer *b, uint64_t add_slots, uint64_t add_objs, uint64_t add_dptrs)
{
    uint64_t const ns = nslots(b) + add_slots;
    uint64_t const no = nobjs(b) + add_objs;
    uint64_t const nd = ndptrs(b) + add_dptrs;
    if (ns <= b->slots_cap && no <= b->objs_cap && nd <= b->dptr_cap) return true;
    uint64_t sc = b->slots_cap, oc = b->objs_cap, dc = b->dptr_cap;
    while (sc < ns) sc = sc ? 2 * sc : 64;
    while (oc < no) oc = oc ? 2 * oc : 16;
    while (dc < nd) dc = dc ? 2 * dc : 16;
    stg::ImageView v;
    std::string err;
    if (!v.open(b->mem, b->cap_words * 8, &err)) {
        set_error(err);
        return false;
    }
    return relayout(b, &v, sc, oc, dc);
}

// Adopt a foreign image: copy it and shift every stored address to the
// new location (the reference's NS(ManagedBuffer_remap)).
st_Buffer *adopt_image(const unsigned char *data, uint64_t size)
{
    stg::ImageView v;
    std::string err;
    if (!v.open(data, size, &err)) {
        set_error(err);
        return nullptr;
    }
    st_Buffer *b = new (std::nothrow) st_Buffer();
    if (!b) return nullptr;
    uint64_t const ns = v.img[v.word_of(v.img[3]) + 1];
    if (!relayout(b, &v, ns + 64, v.num_objects + 16, v.num_dataptrs + 16)) {
        delete b;
        return nullptr;
    }
    return b;
}

}  // namespace

extern "C" {

const char *st_last_error(void) { return stg::g_last_error.c_str(); }

st_Buffer *st_Buffer_new(st_buffer_size_t capacity)
{
    st_Buffer *b = new (std::nothrow) st_Buffer();
    if (!b) return nullptr;
    uint64_t const slots = capacity > 0 ? capacity / 8 + 64 : 64;
    if (!relayout(b, nullptr, slots, 16, 16)) {
        delete b;
        return nullptr;
    }
    return b;
}

st_Buffer *st_Buffer_new_on_data(const unsigned char *data, st_buffer_size_t size)
{
    return adopt_image(data, size);
}

st_Buffer *st_Buffer_new_from_copy(const st_Buffer *other)
{
    if (!other) return nullptr;
    return adopt_image((const unsigned char *)other->mem, other->cap_words * 8);
}

st_Buffer *st_Buffer_new_from_file(const char *path)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        set_error(std::string("cannot open ") + (path ? path : "(null)"));
        return nullptr;
    }
    std::fseek(f, 0, SEEK_END);
    long const n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<unsigned char> data(n > 0 ? (size_t)n : 0);
    size_t const got = n > 0 ? std::fread(data.data(), 1, (size_t)n, f) : 0;
    std::fclose(f);
    if (n <= 0 || got != (size_t)n || n % 8 != 0) {
        set_error("CObjects file is empty or truncated");
        return nullptr;
    }
    std::vector<uint64_t> aligned((size_t)n / 8);
    std::memcpy(aligned.data(), data.data(), (size_t)n);
    return adopt_image((const unsigned char *)aligned.data(), (uint64_t)n);
}

void st_Buffer_delete(st_Buffer *b)
{
    if (!b) return;
    std::free(b->mem);
    delete b;
}

int32_t st_Buffer_write_to_file(const st_Buffer *b, const char *path)
{
    if (!b || !path) return -1;
    FILE *f = std::fopen(path, "wb");
    if (!f) return -1;
    size_t const n = (size_t)b->mem[1];
    size_t const put = std::fwrite(b->mem, 1, n, f);
    std::fclose(f);
    return put == n ? 0 : -1;
}

int32_t st_Buffer_reset(st_Buffer *b)
{
    if (!b) return -1;
    return relayout(b, nullptr, b->slots_cap, b->objs_cap, b->dptr_cap) ? 0 : -1;
}

st_Buffer *st_Buffer_new_detailed(st_buffer_size_t max_num_objects,
                                  st_buffer_size_t max_num_slots,
                                  st_buffer_size_t max_num_dataptrs,
                                  st_buffer_size_t max_num_garbage_ranges, uint64_t flags)
{
    (void)max_num_garbage_ranges;  // no garbage ranges are kept: objects are never freed
    (void)flags;
    st_Buffer *b = new (std::nothrow) st_Buffer();
    if (!b) return nullptr;
    if (!relayout(b, nullptr, max_num_slots, max_num_objects, max_num_dataptrs)) {
        delete b;
        return nullptr;
    }
    return b;
}

int32_t st_Buffer_reserve(st_Buffer *b, st_buffer_size_t max_num_objects,
                          st_buffer_size_t max_num_slots, st_buffer_size_t max_num_dataptrs,
                          st_buffer_size_t max_num_garbage_ranges)
{
    (void)max_num_garbage_ranges;
    if (!b) return -1;
    if (max_num_objects <= b->objs_cap && max_num_slots <= b->slots_cap &&
        max_num_dataptrs <= b->dptr_cap)
        return 0;
    stg::ImageView v;
    std::string err;
    if (!v.open(b->mem, b->cap_words * 8, &err)) {
        set_error(err);
        return -1;
    }
    return relayout(b, &v, std::max<uint64_t>(b->slots_cap, max_num_slots),
                    std::max<uint64_t>(b->objs_cap, max_num_objects),
                    std::max<uint64_t>(b->dptr_cap, max_num_dataptrs))
               ? 0
               : -1;
}

int32_t st_Buffer_reset_detailed(st_Buffer *b, st_buffer_size_t max_num_objects,
                                 st_buffer_size_t max_num_slots,
                                 st_buffer_size_t max_num_dataptrs,
                                 st_buffer_size_t max_num_garbage_ranges)
{
    (void)max_num_garbage_ranges;
    if (!b) return -1;
    return relayout(b, nullptr, max_num_slots, max_num_objects, max_num_dataptrs) ? 0 : -1;
}

int32_t st_Buffer_reserve_capacity(st_Buffer *b, st_buffer_size_t capacity)
{
    if (!b) return -1;
    if (capacity <= b->cap_words * 8) return 0;
    uint64_t const more = (capacity - b->cap_words * 8 + 7) / 8;
    return st_Buffer_reserve(b, b->objs_cap, b->slots_cap + more, b->dptr_cap, 0);
}

int32_t st_Buffer_read_from_file(st_Buffer *b, const char *path)
{
    if (!b) return -1;
    st_Buffer *n = st_Buffer_new_from_file(path);
    if (!n) return -1;
    uint64_t const gen = b->generation;
    std::free(b->mem);
    *b = *n;
    b->generation = gen + 1;
    n->mem = nullptr;
    delete n;
    return 0;
}

// The image with every stored address moved to `norm_base` (header, object
// table, dataptr table, the pointer fields the dataptrs name, and an
// interpolated space-charge kick's table address when it points into the
// buffer), written to `path` (buffer.h:334-337).
int32_t st_Buffer_write_to_file_normalized_addr(const st_Buffer *b, const char *path,
                                                st_buffer_addr_t norm_base)
{
    if (!b || !path) return -1;
    uint64_t const base = base_of(b), size = b->mem[1], nw = size / 8;
    auto inside = [&](uint64_t a) { return a >= base && a < base + size; };
    auto moved = [&](uint64_t a) { return a - base + norm_base; };
    std::vector<uint64_t> img(b->mem, b->mem + nw);
    img[0] = norm_base;
    for (int k = 3; k <= 6; ++k) img[k] = moved(b->mem[k]);
    uint64_t const no = nobjs(b), nd = ndptrs(b);
    for (uint64_t i = 0; i < no; ++i) {
        uint64_t const e = b->objs_w + 2 + 3 * i;
        img[e] = moved(b->mem[e]);
        if (b->mem[e + 1] == ST_OBJECT_TYPE_SC_INTERPOLATED_PROF && b->mem[e + 2] >= 56) {
            uint64_t const w = (b->mem[e] - base) / 8 + 6;
            if (w < nw && inside(b->mem[w])) img[w] = moved(b->mem[w]);
        }
    }
    for (uint64_t k = 0; k < nd; ++k) {
        uint64_t const e = b->dptr_w + 2 + k;
        uint64_t const field = b->mem[e];
        img[e] = moved(field);
        if (inside(field)) {
            uint64_t const w = (field - base) / 8;
            if (w < nw && inside(b->mem[w])) img[w] = moved(b->mem[w]);
        }
    }
    FILE *f = std::fopen(path, "wb");
    if (!f) return -1;
    size_t const put = std::fwrite(img.data(), 1, (size_t)size, f);
    std::fclose(f);
    return put == size ? 0 : -1;
}

int32_t st_Buffer_clear(st_Buffer *b, bool set_data_to_zero)
{
    (void)set_data_to_zero;  // the new layout is zero-filled
    return st_Buffer_reset(b);
}

// A buffer of this library is always mapped at its own address: its stored
// base address equals where it lives, so remapping has nothing to do.
bool st_Buffer_needs_remapping(const st_Buffer *b) { return b && b->mem[0] != base_of(b); }
int32_t st_Buffer_remap(st_Buffer *b) { return (b && !st_Buffer_needs_remapping(b)) ? 0 : -1; }
int32_t st_Buffer_refresh(st_Buffer *b) { return st_Buffer_remap(b); }

st_buffer_size_t st_Buffer_get_header_size(const st_Buffer *b) { return b ? b->mem[2] : 0; }
st_buffer_addr_t st_Buffer_get_data_end_addr(const st_Buffer *b)
{
    return b ? base_of(b) + b->mem[1] : 0;
}
st_buffer_size_t st_Buffer_get_max_num_of_objects(const st_Buffer *b) { return b ? b->objs_cap : 0; }
st_buffer_size_t st_Buffer_get_max_num_of_slots(const st_Buffer *b) { return b ? b->slots_cap : 0; }
st_buffer_size_t st_Buffer_get_max_num_of_dataptrs(const st_Buffer *b) { return b ? b->dptr_cap : 0; }
st_buffer_size_t st_Buffer_get_num_of_garbage_ranges(const st_Buffer *) { return 0; }
st_buffer_size_t st_Buffer_get_max_num_of_garbage_ranges(const st_Buffer *) { return 0; }

st_buffer_size_t st_Buffer_get_size(const st_Buffer *b) { return b ? b->mem[1] : 0; }
st_buffer_size_t st_Buffer_get_capacity(const st_Buffer *b) { return b ? b->cap_words * 8 : 0; }
st_buffer_size_t st_Buffer_get_slot_size(const st_Buffer *b) { return b ? 8 : 0; }
st_buffer_size_t st_Buffer_get_num_of_objects(const st_Buffer *b) { return b ? nobjs(b) : 0; }
st_buffer_size_t st_Buffer_get_num_of_slots(const st_Buffer *b) { return b ? nslots(b) : 0; }
st_buffer_size_t st_Buffer_get_num_of_dataptrs(const st_Buffer *b) { return b ? ndptrs(b) : 0; }
unsigned char *st_Buffer_get_data_begin(st_Buffer *b) { return b ? (unsigned char *)b->mem : nullptr; }
const unsigned char *st_Buffer_get_const_data_begin(const st_Buffer *b)
{
    return b ? (const unsigned char *)b->mem : nullptr;
}
st_buffer_addr_t st_Buffer_get_data_begin_addr(const st_Buffer *b) { return b ? base_of(b) : 0; }

st_Object *st_Buffer_get_objects_begin(st_Buffer *b)
{
    return b ? (st_Object *)(b->mem + b->objs_w + 2) : nullptr;
}
st_Object *st_Buffer_get_objects_end(st_Buffer *b)
{
    return b ? st_Buffer_get_objects_begin(b) + nobjs(b) : nullptr;
}
const st_Object *st_Buffer_get_const_objects_begin(const st_Buffer *b)
{
    return b ? (const st_Object *)(b->mem + b->objs_w + 2) : nullptr;
}
const st_Object *st_Buffer_get_const_objects_end(const st_Buffer *b)
{
    return b ? st_Buffer_get_const_objects_begin(b) + nobjs(b) : nullptr;
}
const st_Object *st_Buffer_get_const_object(const st_Buffer *b, st_buffer_size_t i)
{
    return (b && i < nobjs(b)) ? st_Buffer_get_const_objects_begin(b) + i : nullptr;
}
st_Object *st_Buffer_get_object(st_Buffer *b, st_buffer_size_t i)
{
    return (b && i < nobjs(b)) ? st_Buffer_get_objects_begin(b) + i : nullptr;
}

st_object_type_id_t st_Object_get_type_id(const st_Object *o) { return o ? o->type_id : 0; }
st_buffer_addr_t st_Object_get_begin_addr(const st_Object *o) { return o ? o->begin_addr : 0; }
st_buffer_size_t st_Object_get_size(const st_Object *o) { return o ? o->size : 0; }

void *st_Buffer_add_object(st_Buffer *b, const void *struct_data, st_buffer_size_t struct_size,
                           st_object_type_id_t type_id, st_buffer_size_t num_dataptrs,
                           const st_buffer_size_t *field_word_index,
                           const void *const *array_data, const st_buffer_size_t *array_words)
{
    if (!b || struct_size == 0) return nullptr;
    uint64_t const sw = (struct_size + 7) / 8;
    uint64_t total = sw;
    for (uint64_t k = 0; k < num_dataptrs; ++k) {
        if (field_word_index[k] >= sw) {
            set_error("st_Buffer_add_object: pointer field outside the struct");
            return nullptr;
        }
        total += array_words[k];
    }
    if (!ensure(b, total, 1, num_dataptrs)) return nullptr;
    uint64_t const base = base_of(b);
    uint64_t const pos = b->slots_w + 2 + nslots(b);
    uint64_t *dst = b->mem + pos;
    std::memset(dst, 0, total * 8);
    if (struct_data) std::memcpy(dst, struct_data, (size_t)struct_size);
    uint64_t off = sw;
    for (uint64_t k = 0; k < num_dataptrs; ++k) {
        uint64_t const nw = array_words[k];
        if (array_data && array_data[k] && nw) std::memcpy(dst + off, array_data[k], nw * 8);
        dst[field_word_index[k]] = base + (pos + off) * 8;
        b->mem[b->dptr_w + 2 + ndptrs(b) + k] = base + (pos + field_word_index[k]) * 8;
        off += nw;
    }
    b->mem[b->dptr_w + 1] += num_dataptrs;
    uint64_t const e = b->objs_w + 2 + 3 * nobjs(b);
    b->mem[e] = base + pos * 8;
    b->mem[e + 1] = type_id;
    b->mem[e + 2] = total * 8;
    b->mem[b->objs_w + 1] += 1;
    b->mem[b->slots_w + 1] += total;
    ++b->generation;
    return dst;
}

uint64_t stg_buffer_generation(const st_Buffer *b) { return b ? b->generation : 0; }

}  // extern "C"

st_Buffer *stg::buffer_take_contents(st_Buffer *b)
{
    if (!b) return nullptr;
    st_Buffer *empty = st_Buffer_new(0);
    if (!empty) return nullptr;
    st_Buffer *n = new (std::nothrow) st_Buffer(*b);
    if (!n) {
        st_Buffer_delete(empty);
        return nullptr;
    }
    uint64_t const gen = b->generation;
    *b = *empty;  // b takes the fresh empty layout; `empty` gives up its memory
    b->generation = gen + 1;
    empty->mem = nullptr;
    delete empty;
    return n;
}

// ------------------------------------------------------------ elements
namespace {

template <typename T>
T *add_plain(st_Buffer *b, const T &v, uint64_t type_id)
{
    return static_cast<T *>(
        st_Buffer_add_object(b, &v, sizeof(T), type_id, 0, nullptr, nullptr, nullptr));
}

}  // namespace

extern "C" {

st_Drift *st_Drift_new(st_Buffer *b) { return st_Drift_add(b, 0.0); }
st_Drift *st_Drift_add(st_Buffer *b, double length)
{
    st_Drift d{length};
    return add_plain(b, d, ST_OBJECT_TYPE_DRIFT);
}
st_DriftExact *st_DriftExact_new(st_Buffer *b) { return st_DriftExact_add(b, 0.0); }
st_DriftExact *st_DriftExact_add(st_Buffer *b, double length)
{
    st_DriftExact d{length};
    return add_plain(b, d, ST_OBJECT_TYPE_DRIFT_EXACT);
}

st_Multipole *st_Multipole_new(st_Buffer *b, int64_t order)
{
    return st_Multipole_add(b, order, nullptr, 0.0, 0.0, 0.0);
}
st_Multipole *st_Multipole_add(st_Buffer *b, int64_t order, const double *bal, double length,
                               double hxl, double hyl)
{
    if (order < 0) return nullptr;
    st_Multipole m{order, length, hxl, hyl, 0};
    st_buffer_size_t const field = 4, nw = (st_buffer_size_t)(2 * order + 2);
    const void *arr[1] = {bal};
    return static_cast<st_Multipole *>(st_Buffer_add_object(
        b, &m, sizeof(m), ST_OBJECT_TYPE_MULTIPOLE, 1, &field, arr, &nw));
}
double *st_Multipole_bal(st_Multipole *mp)
{
    return mp ? (double *)(uintptr_t)mp->bal_addr : nullptr;
}

st_RFMultipole *st_RFMultipole_new(st_Buffer *b, int64_t order)
{
    return st_RFMultipole_add(b, order, 0.0, 0.0, 0.0, nullptr, nullptr);
}
st_RFMultipole *st_RFMultipole_add(st_Buffer *b, int64_t order, double voltage,
                                   double frequency, double lag, const double *bal,
                                   const double *phase)
{
    if (order < 0) return nullptr;
    st_RFMultipole m{order, voltage, frequency, lag, 0, 0};
    st_buffer_size_t const fields[2] = {4, 5};
    st_buffer_size_t const nw[2] = {(st_buffer_size_t)(2 * order + 2),
                                    (st_buffer_size_t)(2 * order + 2)};
    const void *arr[2] = {bal, phase};
    return static_cast<st_RFMultipole *>(st_Buffer_add_object(
        b, &m, sizeof(m), ST_OBJECT_TYPE_RF_MULTIPOLE, 2, fields, arr, nw));
}

st_Cavity *st_Cavity_new(st_Buffer *b) { return st_Cavity_add(b, 0.0, 0.0, 0.0); }
st_Cavity *st_Cavity_add(st_Buffer *b, double voltage, double frequency, double lag)
{
    st_Cavity c{voltage, frequency, lag};
    return add_plain(b, c, ST_OBJECT_TYPE_CAVITY);
}
st_XYShift *st_XYShift_new(st_Buffer *b) { return st_XYShift_add(b, 0.0, 0.0); }
st_XYShift *st_XYShift_add(st_Buffer *b, double dx, double dy)
{
    st_XYShift s{dx, dy};
    return add_plain(b, s, ST_OBJECT_TYPE_XYSHIFT);
}
st_SRotation *st_SRotation_new(st_Buffer *b) { return st_SRotation_add_detailed(b, 1.0, 0.0); }
st_SRotation *st_SRotation_add(st_Buffer *b, double angle)
{
    return st_SRotation_add_detailed(b, std::cos(angle), std::sin(angle));
}
st_SRotation *st_SRotation_add_detailed(st_Buffer *b, double cos_z, double sin_z)
{
    st_SRotation r{cos_z, sin_z};
    return add_plain(b, r, ST_OBJECT_TYPE_SROTATION);
}
st_LimitRect *st_LimitRect_new(st_Buffer *b) { return st_LimitRect_add(b, -1.0, 1.0, -1.0, 1.0); }
st_LimitRect *st_LimitRect_add(st_Buffer *b, double min_x, double max_x, double min_y,
                               double max_y)
{
    st_LimitRect l{min_x, max_x, min_y, max_y};
    return add_plain(b, l, ST_OBJECT_TYPE_LIMIT_RECT);
}
st_LimitEllipse *st_LimitEllipse_new(st_Buffer *b) { return st_LimitEllipse_add(b, 1.0, 1.0); }
st_LimitEllipse *st_LimitEllipse_add(st_Buffer *b, double a, double bb)
{
    st_LimitEllipse l{a * a, bb * bb, (a * a) * (bb * bb)};
    return add_plain(b, l, ST_OBJECT_TYPE_LIMIT_ELLIPSE);
}
st_LimitRectEllipse *st_LimitRectEllipse_new(st_Buffer *b)
{
    return st_LimitRectEllipse_add(b, 1.0, 1.0, 1.0, 1.0);
}
st_LimitRectEllipse *st_LimitRectEllipse_add(st_Buffer *b, double max_x, double max_y,
                                             double a_squ, double b_squ)
{
    st_LimitRectEllipse l{max_x, max_y, a_squ, b_squ, a_squ * b_squ};
    return add_plain(b, l, ST_OBJECT_TYPE_LIMIT_RECT_ELLIPSE);
}
st_DipoleEdge *st_DipoleEdge_new(st_Buffer *b) { return st_DipoleEdge_add(b, 0.0, 0.0); }
st_DipoleEdge *st_DipoleEdge_add(st_Buffer *b, double r21, double r43)
{
    st_DipoleEdge d{r21, r43};
    return add_plain(b, d, ST_OBJECT_TYPE_DIPEDGE);
}
st_BeamMonitor *st_BeamMonitor_new(st_Buffer *b)
{
    return st_BeamMonitor_add(b, 0, 0, 1, 0, 0, 0, false, true);
}
st_BeamMonitor *st_BeamMonitor_add(st_Buffer *b, int64_t num_stores, int64_t start,
                                   int64_t skip, st_buffer_addr_t out_address,
                                   int64_t min_particle_id, int64_t max_particle_id,
                                   bool is_rolling, bool is_turn_ordered)
{
    st_BeamMonitor m{num_stores, start, skip, out_address, max_particle_id,
                     min_particle_id, is_rolling ? 1 : 0, is_turn_ordered ? 1 : 0};
    return add_plain(b, m, ST_OBJECT_TYPE_BEAM_MONITOR);
}

static void *add_data_element(st_Buffer *b, uint64_t type, st_buffer_size_t n,
                              const double *data)
{
    st_BeamBeam4D e{n, 0};
    st_buffer_size_t const field = 1;
    const void *arr[1] = {data};
    return st_Buffer_add_object(b, &e, sizeof(e), type, 1, &field, arr, &n);
}
st_BeamBeam4D *st_BeamBeam4D_new(st_Buffer *b, st_buffer_size_t n)
{
    return st_BeamBeam4D_add(b, n, nullptr);
}
st_BeamBeam4D *st_BeamBeam4D_add(st_Buffer *b, st_buffer_size_t n, const double *data)
{
    return (st_BeamBeam4D *)add_data_element(b, ST_OBJECT_TYPE_BEAM_BEAM_4D, n, data);
}
st_BeamBeam6D *st_BeamBeam6D_new(st_Buffer *b, st_buffer_size_t n)
{
    return st_BeamBeam6D_add(b, n, nullptr);
}
st_BeamBeam6D *st_BeamBeam6D_add(st_Buffer *b, st_buffer_size_t n, const double *data)
{
    return (st_BeamBeam6D *)add_data_element(b, ST_OBJECT_TYPE_BEAM_BEAM_6D, n, data);
}
st_SCCoasting *st_SCCoasting_new(st_Buffer *b)
{
    return st_SCCoasting_add(b, 0.0, 1.0, 1.0, 1.0, 0.0, 0.0, 0.0, 1e-10, true);
}
st_SCCoasting *st_SCCoasting_add(st_Buffer *b, double n, double circ, double sx, double sy,
                                 double length, double x_co, double y_co, double msd,
                                 bool enabled)
{
    st_SCCoasting e{n, circ, sx, sy, length, x_co, y_co, msd, enabled ? 1u : 0u};
    return add_plain(b, e, ST_OBJECT_TYPE_SC_COASTING);
}
st_SCQGaussProfile *st_SCQGaussProfile_new(st_Buffer *b)
{
    return st_SCQGaussProfile_add(b, 0.0, 1.0, 1.0, 1.0, 0.0, 0.0, 0.0, 1e-10, 1.0, true);
}
st_SCQGaussProfile *st_SCQGaussProfile_add(st_Buffer *b, double n, double blen, double sx,
                                           double sy, double length, double x_co,
                                           double y_co, double msd, double q, bool enabled)
{
    // cq: normalisation of the q-Gaussian (internal/math_qgauss.h:140-165)
    double cq = std::sqrt(M_PI);
    double const eps = 1e-6;
    if (q >= 1.0 + eps) {
        cq *= std::tgamma((3.0 - q) / (2.0 * (q - 1.0)));
        cq /= std::sqrt(q - 1.0) * std::tgamma(1.0 / (q - 1.0));
    } else if (q <= 1.0 - eps) {
        cq *= 2.0 * std::tgamma(1.0 / (1.0 - q));
        cq /= (3.0 - q) * std::sqrt(1.0 - q) * std::tgamma((3.0 - q) / (2.0 * (1.0 - q)));
    }
    st_SCQGaussProfile e{n, blen, sx, sy, length, x_co, y_co, msd, q, cq, enabled ? 1u : 0u};
    return add_plain(b, e, ST_OBJECT_TYPE_SC_QGAUSSIAN_PROF);
}

// ------------------------------------------------------------ particles
st_Particles *st_Particles_new(st_Buffer *b, st_buffer_size_t n)
{
    uint64_t st[22];
    std::memset(st, 0, sizeof(st));
    st[0] = n;
    st_buffer_size_t fields[21], nw[21];
    for (int c = 0; c < 21; ++c) {
        fields[c] = (st_buffer_size_t)(1 + c);
        nw[c] = n;
    }
    return static_cast<st_Particles *>(st_Buffer_add_object(
        b, st, sizeof(st), ST_OBJECT_TYPE_PARTICLE, 21, fields, nullptr, nw));
}

st_Particles *st_Particles_add_copy(st_Buffer *b, const st_Particles *o)
{
    if (!o) return nullptr;
    st_Particles *p = st_Particles_new(b, (st_buffer_size_t)o->num_particles);
    if (p) st_Particles_copy(p, o);
    return p;
}

st_Particles *st_Particles_buffer_get_particles(st_Buffer *b, st_buffer_size_t index)
{
    st_Object *o = st_Buffer_get_object(b, index);
    if (!o || o->type_id != ST_OBJECT_TYPE_PARTICLE) return nullptr;
    return (st_Particles *)(uintptr_t)o->begin_addr;
}
const st_Particles *st_Particles_buffer_get_const_particles(const st_Buffer *b,
                                                            st_buffer_size_t index)
{
    const st_Object *o = st_Buffer_get_const_object(b, index);
    if (!o || o->type_id != ST_OBJECT_TYPE_PARTICLE) return nullptr;
    return (const st_Particles *)(uintptr_t)o->begin_addr;
}
int64_t st_Particles_get_num_of_particles(const st_Particles *p) { return p ? p->num_particles : 0; }
st_buffer_size_t st_Particles_buffer_get_num_of_particle_blocks(const st_Buffer *b)
{
    st_buffer_size_t n = 0;
    for (const st_Object *o = st_Buffer_get_const_objects_begin(b);
         o != st_Buffer_get_const_objects_end(b); ++o)
        if (o->type_id == ST_OBJECT_TYPE_PARTICLE) ++n;
    return n;
}

void st_Particles_set_reference(st_Particles *p, double p0c, double mass0, double q0)
{
    if (!p) return;
    double const e0 = std::sqrt(p0c * p0c + mass0 * mass0);
    for (int64_t i = 0; i < p->num_particles; ++i) {
        p->q0[i] = q0;
        p->mass0[i] = mass0;
        p->p0c[i] = p0c;
        p->beta0[i] = p0c / e0;
        p->gamma0[i] = e0 / mass0;
    }
}

// NS(Particles_update_delta_value): particles.h:5459-5496
void st_Particles_update_delta_value(st_Particles *p, int64_t i, double nd)
{
    if (!p || i < 0 || i >= p->num_particles) return;
    double const beta0 = p->beta0[i];
    double const db0 = nd * beta0;
    double const ptau_beta0 = std::sqrt(db0 * db0 + 2.0 * db0 * beta0 + 1.0) - 1.0;
    double const opd = 1.0 + nd;
    p->delta[i] = nd;
    p->rvv[i] = opd / (1.0 + ptau_beta0);
    p->rpp[i] = 1.0 / opd;
    p->psigma[i] = ptau_beta0 / (beta0 * beta0);
}

int32_t st_Particles_copy(st_Particles *d, const st_Particles *s)
{
    if (!d || !s || d->num_particles != s->num_particles) return -1;
    size_t const n = (size_t)s->num_particles * 8;
    double *const *dr = &d->q0;
    double *const *sr = &s->q0;
    for (int c = 0; c < 17; ++c) std::memcpy(dr[c], sr[c], n);
    int64_t *const *di = &d->particle_id;
    int64_t *const *si = &s->particle_id;
    for (int c = 0; c < 4; ++c) std::memcpy(di[c], si[c], n);
    return 0;
}

// ------------------------------------------------------ elem-by-elem config
int32_t st_ElemByElemConfig_init_detailed(st_ElemByElemConfig *c, int64_t order,
                                          int64_t min_pid, int64_t max_pid, int64_t min_elem,
                                          int64_t max_elem, int64_t min_turn,
                                          int64_t max_turn, bool is_rolling)
{
    if (!c || order != 0 || min_pid < 0 || max_pid < min_pid || min_elem < 0 ||
        max_elem < min_elem || min_turn < 0 || max_turn < min_turn)
        return -1;
    c->order = order;
    c->min_particle_id = min_pid;
    c->max_particle_id = max_pid;
    c->min_element_id = min_elem;
    c->max_element_id = max_elem;
    c->min_turn = min_turn;
    c->max_turn = max_turn;
    c->num_particles_to_store = max_pid - min_pid + 1;
    c->num_elements_to_store = max_elem - min_elem + 1;
    c->num_turns_to_store = max_turn - min_turn + 1;
    c->is_rolling = is_rolling ? 1 : 0;
    c->out_store_addr = 0;
    return 0;
}

// output/elem_by_elem_config.h:667-763
int64_t st_ElemByElemConfig_get_particles_store_index_details(const st_ElemByElemConfig *c,
                                                               int64_t pid, int64_t elem,
                                                               int64_t turn)
{
    int64_t out = -1;
    if (!c) return out;
    if (c->min_particle_id <= pid && c->max_particle_id >= pid && c->min_element_id <= elem &&
        c->max_element_id >= elem && c->min_turn <= turn &&
        (c->max_turn >= turn || c->is_rolling != 0)) {
        int64_t const np = c->num_particles_to_store, ne = c->num_elements_to_store;
        int64_t cap = 0;
        if (c->order == 0) {
            out = (turn - c->min_turn) * np * ne + (elem - c->min_element_id) * np +
                  (pid - c->min_particle_id);
            cap = np * ne * c->num_turns_to_store;
        }
        if (out >= cap && cap > 0 && c->is_rolling != 0) out = out % cap;
    }
    return out;
}

int64_t st_ElemByElemConfig_get_stored_num_particles(const st_ElemByElemConfig *c)
{
    return c ? c->num_particles_to_store * c->num_elements_to_store * c->num_turns_to_store : 0;
}

}  // extern "C"

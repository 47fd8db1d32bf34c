// common.h -- internal helpers shared by the host-side translation units.
#pragma once

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "sixtracklib_gb300.h"

namespace stg {

// Per-thread last-error message, read through st_last_error().
void set_error(const std::string &msg);
void clear_error();

// A new st_Buffer holding b's contents (same memory, so object addresses
// are unchanged); b is left a valid empty buffer.  Null on failure, with b
// untouched (buffer.hpp: MAKE_FROM_CBUFFER_AND_TAKE_OWNERSHIP).
st_Buffer *buffer_take_contents(st_Buffer *b);

inline double w2d(uint64_t w)
{
    double d;
    std::memcpy(&d, &w, 8);
    return d;
}
inline uint64_t d2w(double d)
{
    uint64_t w;
    std::memcpy(&w, &d, 8);
    return w;
}

// A read-only view of a CObjects image.  All stored addresses are resolved
// relative to the stored base address (header word 0), so the view works on
// images at any memory location, remapped or not.
struct ImageView {
    const uint64_t *img = nullptr;
    uint64_t base = 0;
    uint64_t size_words = 0;
    const uint64_t *objs = nullptr;  // 3 words per object
    uint64_t num_objects = 0;
    const uint64_t *dptrs = nullptr;
    uint64_t num_dataptrs = 0;

    bool open(const void *image, uint64_t max_bytes, std::string *err);
    // Word offset of an absolute stored address, or UINT64_MAX if outside.
    uint64_t word_of(uint64_t addr) const
    {
        if (addr < base) return UINT64_MAX;
        uint64_t off = addr - base;
        if (off % 8 != 0 || off / 8 >= size_words) return UINT64_MAX;
        return off / 8;
    }
    uint64_t type_of(uint64_t i) const { return objs[3 * i + 1]; }
    uint64_t begin_word(uint64_t i) const { return word_of(objs[3 * i]); }
    uint64_t size_bytes(uint64_t i) const { return objs[3 * i + 2]; }
    const uint64_t *words(uint64_t i) const { return img + begin_word(i); }
    // Pointer field f of object i resolved to a word pointer (or null).
    const uint64_t *deref(uint64_t i, uint64_t field) const
    {
        uint64_t w = word_of(words(i)[field]);
        return (w == UINT64_MAX) ? nullptr : img + w;
    }
};

}  // namespace stg

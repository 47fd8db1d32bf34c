// lattice_view.h -- what a launch needs to know about an st_DeviceLattice,
// for entry points outside engine.cu.
#pragma once

#include <cstdint>

#include "sixtracklib_gb300.h"

namespace stg {

struct LatticeLaunchView {
    const uint64_t *stream = nullptr;  // device: chunked element stream
    const double *s_table = nullptr;   // device: s table
    int32_t n_chunks = 0, chunk_words = 0, stages = 0;
    int32_t threads = 0, blocks_per_sm = 1;
    int64_t num_elements = 0;
    bool fast = false;
    uint64_t xlim_bits = 0, ylim_bits = 0;
    int device = 0;
    const int64_t *elem_offset = nullptr;  // device: record offset per element
    uint32_t op_mask = 0;                  // opcodes present in the lattice
};

bool device_lattice_view(const st_DeviceLattice *lat, LatticeLaunchView *view);
uint64_t *device_scratch(int device, int64_t words);
// Order work on `stream` that uses device_scratch() after the previous work
// that used it (any stream), and mark the end of this work: begin before the
// first launch that touches the scratch, end after the last one.
bool shared_scratch_begin(int device, void *stream);
void shared_scratch_end(int device, void *stream);
void count_launches(uint64_t n);

}  // namespace stg

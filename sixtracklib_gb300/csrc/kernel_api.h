// kernel_api.h -- parameters shared between the host engine and the kernels.
#pragma once

#include <cstdint>

#include "stream.h"

namespace stg {

constexpr int kMaxThreads = 256;  // largest block the kernels are built for
constexpr int kDefaultStages = 4;

enum TrackMode : int32_t { MODE_UNTIL = 0, MODE_LINE = 1, MODE_EBE = 2 };

enum ErrorBits : int32_t { ERR_PIPELINE_TIMEOUT = 1 };

// Opcodes of the plain-ring kernel instantiation: drifts, multipoles,
// shifts, rotations, dipole edges, cavities, apertures and monitors.  A
// lattice with none of the beam-field, space-charge or RF-multipole maps is
// tracked by a kernel compiled without them, which needs fewer registers
// (no spills at two CTAs per SM) and keeps the dispatch switch short.
constexpr uint32_t kPlainOps =
    (1u << OP_END) | (1u << OP_DRIFT) | (1u << OP_DRIFT_EXACT) | (1u << OP_MULTIPOLE) |
    (1u << OP_MULTIPOLE_CURV) | (1u << OP_CAVITY) | (1u << OP_XYSHIFT) | (1u << OP_SROTATION) |
    (1u << OP_LIMIT_RECT) | (1u << OP_LIMIT_ELLIPSE) | (1u << OP_LIMIT_RECT_ELLIPSE) |
    (1u << OP_DIPEDGE) | (1u << OP_MONITOR) | (1u << OP_NOP) | (1u << OP_FAIL) |
    (1u << OP_FAIL_LOST);

inline bool plain_lattice(uint32_t op_mask) { return (op_mask & ~kPlainOps) == 0u; }

struct EbeDevConfig {
    int64_t order;
    int64_t num_particles_to_store, num_elements_to_store, num_turns_to_store;
    int64_t min_particle_id, min_element_id, min_turn;
    int64_t max_particle_id, max_element_id, max_turn;
    int64_t is_rolling;
};

struct TrackParams {
    const uint64_t *stream;  // device: n_chunks * chunk_words words
    int32_t n_chunks;
    int32_t chunk_words;
    int32_t stages;
    int32_t mode;
    int64_t num_elements;    // elements in the compiled range
    uint64_t *cols;          // device: 21 x n column block
    int64_t n;
    int64_t i0, i1;          // particle index range
    int64_t until_turn;
    int32_t finish_turn;
    int32_t turn_cap;        // MODE_UNTIL: a block stops after this many turns (0: none)
    uint64_t xlim_bits, ylim_bits;  // global aperture limits as IEEE bits
    int32_t *status;         // device: OR of per-particle status
    int32_t *error;          // device: ErrorBits
    uint64_t *ebe_out;       // device: elem-by-elem column block
    int64_t ebe_cap;
    EbeDevConfig ebe;
    const int64_t *idx;      // device: particle indices to track (null: i0..i1)
    const int64_t *count;    // device: number of entries of idx
    const double *s_table;   // device: s before element k when a turn starts at s = 0
    uint32_t op_mask;        // opcodes present in the compiled range (stream.h)
};

// Launch one tracking kernel on `stream` (a cudaStream_t).  Returns the CUDA
// error code of the launch (0 on success).
// blocks_per_sm selects the register tier: 1 (up to 255 registers, no
// spills) or 2 (at most 128 registers per thread, two CTAs per SM).
// prm.op_mask selects the instantiation: the plain-ring kernel when every
// opcode present is in kPlainOps, the full kernel otherwise.
int launch_track(const TrackParams &prm, bool fast, int threads, int blocks_per_sm,
                 void *stream);
size_t track_smem_bytes(int stages, int chunk_words);

// TriCub cell coefficients (tricub.cu): from the node table `nodes` (8
// values per node of an nx x ny x nz grid) into `cells` (64 per cell), on
// `stream`.  Returns the CUDA error code of the launch.
int launch_tricub_cells(const double *nodes, double *cells, int64_t nx, int64_t ny, int64_t nz,
                        void *stream);

// The fast policy's exponential (maps.cuh exp_fast) on n device values.
int launch_exp_fast(const double *x, double *y, int64_t n, void *stream);
// The fast arithmetic policy's reciprocal (maps.cuh rcp_fast) on n values.
int launch_rcp_fast(const double *x, double *y, int64_t n, void *stream);

// Batched tracking (track_kernel.cu): a work item is a tile of particles of
// one lattice variant, starting at particle `first`.
struct BatchItem {
    int32_t variant;
    int32_t pad_;
    int64_t first;
};

struct BatchLaunch {
    const TrackParams *variants;  // device: one per variant (mode MODE_UNTIL)
    const BatchItem *items;       // device: longest first
    int32_t num_items;
    int32_t *counter;             // device: zero before the launch
    const int64_t *base_turn;     // device: until_turn = *base_turn + turn_offset
    int64_t turn_offset;
    bool fast;
    bool plain;                   // every variant is a plain ring (kPlainOps)
    int threads, blocks_per_sm;
    unsigned grid;
    size_t smem;
};

// Set the kernel's shared-memory limit to `smem` and report how many CTAs
// of `threads` fit on one SM.  Returns the CUDA error code.
int batch_ctas_per_sm(bool fast, bool plain, int threads, int blocks_per_sm, size_t smem,
                      int *per_sm);
int launch_batch(const BatchLaunch &b, void *stream);

// Stable selection of the particles with work left (compact.cu): fills
// idx / count inside `scratch` (select_scratch_words(i1 - i0) words).
int64_t select_scratch_words(int64_t count);
int launch_select(const uint64_t *cols, int64_t n, int64_t i0, int64_t i1, int mode,
                  int64_t until, uint64_t *scratch, int64_t **idx_out, int64_t **count_out,
                  void *stream);

}  // namespace stg

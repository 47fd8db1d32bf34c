// lattice.h -- compile a CObjects lattice into the device element stream.
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "common.h"
#include "stream.h"

namespace stg {

// Per-map feature setting, as SIXTRL_TRACK_MAP_{DISABLED, SKIP, ENABLED}:
// a disabled map fails (the particle is lost), a skipped one does nothing.
enum MapFlag : int { MAP_DISABLED = 0, MAP_SKIP = 1, MAP_ENABLED = 2 };

struct CompileOptions {
    // Global aperture after Drift/DriftExact (SIXTRL_APERTURE_CHECK_AT_DRIFT):
    // 2 always (reference default), 1 if length >= min_length, 0 never.
    int aperture_mode = 2;
    // SIXTRL_TRACK_BEAMBEAM4D / _BEAMBEAM6D / _SPACECHARGE / _TRICUB, with
    // the reference's default build values (Settings.cmake.default)
    int track_bb4d = MAP_ENABLED;
    int track_bb6d = MAP_ENABLED;
    int track_sc = MAP_ENABLED;
    int track_tricub = MAP_DISABLED;
    double aperture_min_length = 0.0;
    int32_t min_chunk_words = 1024;
    // Output slot for the k-th BeamMonitor of the compiled range (element
    // index given): returns {device pointer to a column block, capacity};
    // {0, 0} disables storing for that monitor.
    std::function<std::pair<uint64_t, int64_t>(uint64_t elem_index)> monitor_output;
};

struct CompiledStream {
    std::vector<uint64_t> words;  // num_chunks * chunk_words
    StreamInfo info;
    std::vector<uint64_t> monitor_elements;  // element indices of monitors
    // s_table[k] = s before element k for a turn that starts at s = +0:
    // the drift lengths summed in lattice order, in double, exactly as the
    // tracking loop accumulates them (num_elements + 1 entries).
    std::vector<double> s_table;
    // word offset of each element's record in `words` (num_elements entries)
    std::vector<int64_t> elem_offset;
    // Data kept out of the records (the line-density tables of interpolated
    // space charge): records stay small, so the chunk size -- and with it
    // the shared memory of every stage -- does not grow with a table.  The
    // uploader places `side` in device memory and writes its address plus
    // the offset into each word listed in `side_fixups` ({word index in
    // `words`, offset in `side` in words}).
    std::vector<uint64_t> side;
    std::vector<std::pair<uint64_t, uint64_t>> side_fixups;
    // Device-only words after `side` (offsets continue those of `side`):
    // the TriCub cell coefficient tables, which the uploader computes on the
    // GPU from the node tables in `side` (one entry per distinct TriCubData).
    uint64_t side_device_words = 0;
    struct TricubTable {
        uint64_t nodes;  // offset of the node table in `side` (8 values per node)
        uint64_t cells;  // offset of the cell table (64 coefficients per cell)
        int64_t nx, ny, nz;
    };
    std::vector<TricubTable> tricub_tables;
};

// Compile elements [begin, end) of the image.  Returns false (and sets the
// error text) on malformed elements.
bool compile_lattice(const ImageView &img, uint64_t begin, uint64_t end,
                     const CompileOptions &opt, CompiledStream *out, std::string *err);

}  // namespace stg

// noalloc.cu -- until-turn tracking of device-resident particles without
// allocating memory on the call path.
//
// Some callers cannot call cudaMalloc while they track: code running inside
// another framework's memory management (a PyTorch or JAX operator whose
// buffers all come from the framework's caching allocator, which must not be
// bypassed), or a real-time loop that was given a fixed device-memory budget
// up front.  st_DeviceLattice_track_until allocates on first use (the
// particle-selection scratch grows with the particle count, and the status
// words come from cudaMalloc).  This file provides the same computation with
// that scratch in a file-scope __device__ array instead:
//
//   * capacity: at most kNoAllocMaxParticles particles per call; larger
//     calls are rejected with an error, nothing is launched;
//   * the array exists once per GPU that loads the library and is held until
//     the process exits (about 8 MiB);
//   * every call on a GPU shares the array and it keeps the previous call's
//     contents; the status words are cleared at the start of each call, the
//     selection buffers are fully rewritten before they are read.  Calls that
//     overlap on the same GPU (different streams or threads) race on it and
//     must be serialised by the caller;
//   * the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress (a host-side stand-in is all the name gives host
//     code); make that first call before capturing a stream.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "common.h"
#include "device_guard.h"
#include "kernel_api.h"
#include "lattice_view.h"

namespace stg {

namespace {

constexpr int64_t kNoAllocMaxParticles = 1 << 20;
constexpr int64_t kFlagWords = 32;  // status + error words, padded to 256 B
constexpr int64_t kSelBlocks = (kNoAllocMaxParticles + 1023) / 1024;
constexpr int64_t kSelWords = (kSelBlocks + 1) / 2 + kSelBlocks + 1 + kNoAllocMaxParticles + 4;
constexpr int64_t kNoAllocWords = kFlagWords + kSelWords;

}  // namespace

// The scratch: status words, then the particle-selection buffers.
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocWords];

namespace {

std::mutex g_mu;
uint64_t *g_addr[64] = {};

// Device address of g_noalloc_scratch on `device` (set-up, once per device,
// with that device current).
uint64_t *scratch_address(int device)
{
    if (device < 0 || device >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void *ptr = nullptr;
        cudaError_t const rc = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (rc != cudaSuccess) {
            set_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(rc));
            return nullptr;
        }
        g_addr[device] = static_cast<uint64_t *>(ptr);
    }
    return g_addr[device];
}

}  // namespace

}  // namespace stg

using namespace stg;

extern "C" st_track_status_t st_DeviceLattice_track_until_noalloc(st_DeviceLattice *lat,
                                                                   void *d_cols,
                                                                   int64_t num_particles,
                                                                   int64_t until_turn,
                                                                   void *stream)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    LatticeLaunchView v;
    if (!device_lattice_view(lat, &v)) {
        set_error("st_DeviceLattice_track_until_noalloc: invalid lattice");
        return -1;
    }
    if (num_particles < 0 || num_particles > kNoAllocMaxParticles) {
        set_error("st_DeviceLattice_track_until_noalloc: at most 1048576 particles per call");
        return -1;
    }
    if (num_particles == 0) return 0;
    if (!d_cols) {
        set_error("st_DeviceLattice_track_until_noalloc: null particle columns");
        return -1;
    }
    if (v.num_elements == 0) {  // track/track.h:617: an empty lattice fails
        set_error("st_DeviceLattice_track_until_noalloc: empty lattice");
        return -1;
    }
    cudaError_t rc = cudaSetDevice(v.device);
    if (rc != cudaSuccess) {
        set_error(std::string("cudaSetDevice: ") + cudaGetErrorString(rc));
        return -1;
    }
    uint64_t *base = scratch_address(v.device);
    if (!base) return -1;
    int32_t *flags = reinterpret_cast<int32_t *>(base);
    uint64_t *sel = base + kFlagWords;
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    uint64_t *cols = static_cast<uint64_t *>(d_cols);

    rc = cudaMemsetAsync(flags, 0, 2 * sizeof(int32_t), s);  // status and error start at 0
    if (rc != cudaSuccess) {
        set_error(std::string("cudaMemsetAsync: ") + cudaGetErrorString(rc));
        return -1;
    }
    int64_t *idx = nullptr, *count = nullptr;
    int const rs = launch_select(cols, num_particles, 0, num_particles, MODE_UNTIL, until_turn,
                                 sel, &idx, &count, stream);
    if (rs != 0) {
        set_error(std::string("particle selection launch: ") + cudaGetErrorString((cudaError_t)rs));
        return -1;
    }
    TrackParams prm{};
    prm.stream = v.stream;
    prm.n_chunks = v.n_chunks;
    prm.chunk_words = v.chunk_words;
    prm.stages = v.stages;
    prm.mode = MODE_UNTIL;
    prm.num_elements = v.num_elements;
    prm.cols = cols;
    prm.n = num_particles;
    prm.i0 = 0;
    prm.i1 = num_particles;
    prm.until_turn = until_turn;
    prm.xlim_bits = v.xlim_bits;
    prm.ylim_bits = v.ylim_bits;
    prm.status = flags;
    prm.error = flags + 1;
    prm.idx = idx;
    prm.count = count;
    prm.s_table = v.s_table;
    prm.op_mask = v.op_mask;
    int const rt = launch_track(prm, v.fast, v.threads, v.blocks_per_sm, stream);
    if (rt != 0) {
        set_error(std::string("track kernel launch: ") + cudaGetErrorString((cudaError_t)rt));
        return -1;
    }
    int32_t host_flags[2] = {0, 0};
    rc = cudaMemcpyAsync(host_flags, flags, sizeof(host_flags), cudaMemcpyDeviceToHost, s);
    if (rc == cudaSuccess) rc = cudaStreamSynchronize(s);
    if (rc != cudaSuccess) {
        set_error(std::string("track kernel: ") + cudaGetErrorString(rc));
        return -1;
    }
    if (host_flags[1] != 0) {
        set_error("track kernel: a shared-memory pipeline wait timed out; the blocks that timed "
                  "out left their particles unchanged, other blocks (and earlier launches of "
                  "the call) may have advanced theirs");
        return -1;
    }
    return host_flags[0];
}

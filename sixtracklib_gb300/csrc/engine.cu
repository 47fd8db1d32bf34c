// engine.cu -- host engine: devices, device lattices, particle transfers,
// the free tracking calls and the TrackJob (common/track/track.c:21-141,
// common/internal/track_job.cpp:47-186,417-445, cuda/track/track_job.cpp).
//
// Data on the GPU:
//   * particle sets: one 21 x n column block (NS(Particles) field order),
//     all sets of a job concatenated, resident between calls;
//   * lattice: the compiled element stream (lattice.cpp), chunked for the
//     kernel's shared-memory stages;
//   * outputs: one column block per output Particles object (elem-by-elem
//     store, one per BeamMonitor), written by the kernel in place.
// Every call runs on the GPU; without a usable device the calls fail and
// st_last_error() names the reason.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "common.h"
#include "kernel_api.h"
#include "device_guard.h"
#include "lattice.h"

extern "C" uint64_t stg_buffer_generation(const st_Buffer *b);

namespace stg {

// ------------------------------------------------------------- options
struct Options {
    bool fast = false;
    int threads = 128;           // tracking kernel's block size (effective)
    int threads_general = 128;   // the reference's cuda.threads_per_block
    int track_threads_req = 0;   // cuda.track_threads_per_block as given (0: unset)
    int device = 0;
    int aperture_mode = 2;
    double aperture_min_length = 0.0;
    double x_limit = 1.0, y_limit = 1.0;
    int stages = kDefaultStages;
    int chunk_words = 1024;
    int blocks_per_sm = 2;
    // SIXTRL_TRACK_BEAMBEAM4D / _BEAMBEAM6D / _SPACECHARGE / _TRICUB
    int track_bb4d = MAP_ENABLED, track_bb6d = MAP_ENABLED, track_sc = MAP_ENABLED;
    int track_tricub = MAP_DISABLED;
};

// "enabled" | "skip" | "disabled" (python/sixtracklib/config.py.template)
static int map_flag(const std::string &v)
{
    if (v == "enabled") return MAP_ENABLED;
    if (v == "skip") return MAP_SKIP;
    if (v == "disabled" || v == "disable") return MAP_DISABLED;
    throw std::invalid_argument(v);
}

static std::string trim(const std::string &s)
{
    size_t a = s.find_first_not_of(" \t\r\n\"'");
    size_t b = s.find_last_not_of(" \t\r\n\"'");
    return (a == std::string::npos) ? std::string() : s.substr(a, b - a + 1);
}

// Accepts "key=value" pairs separated by whitespace, ';' or newlines, and
// the reference's TOML form ("[cuda]" sections, "key = value" lines,
// cuda/track/track_job.cpp:1775-1830).
static bool parse_options(const char *cfg, Options *o, std::string *err)
{
    if (!cfg) return true;
    std::string s(cfg);
    for (char &c : s)
        if (c == ';' || c == ',') c = '\n';
    std::istringstream in(s);
    std::string line;
    while (std::getline(in, line)) {
        line = trim(line);
        if (line.empty() || line[0] == '[' || line[0] == '#') continue;
        // allow several key=value pairs on one line
        std::vector<std::string> items;
        std::string cur;
        std::istringstream ws(line);
        std::string tok;
        while (ws >> tok) {
            if (tok == "=" || (!cur.empty() && cur.back() == '=')) {
                cur += tok;
            } else if (!cur.empty() && tok[0] == '=') {
                cur += tok;
            } else {
                if (!cur.empty()) items.push_back(cur);
                cur = tok;
            }
        }
        if (!cur.empty()) items.push_back(cur);
        for (const std::string &it : items) {
            size_t const eq = it.find('=');
            if (eq == std::string::npos) {
                if (err) *err = "config: expected key=value, got '" + it + "'";
                return false;
            }
            std::string k = trim(it.substr(0, eq));
            std::string const v = trim(it.substr(eq + 1));
            if (k.rfind("cuda.", 0) == 0) k = k.substr(5);  // dotted TOML keys
            try {
                if (k == "mode") {
                    if (v == "fast") o->fast = true;
                    else if (v == "exact") o->fast = false;
                    else throw std::invalid_argument(v);
                } else if (k == "threads_per_block" || k == "threads") {
                    o->threads_general = std::stoi(v);
                } else if (k == "track_threads_per_block") {
                    o->track_threads_req = std::stoi(v);
                } else if (k == "device" || k == "device_id") {
                    o->device = std::stoi(v);
                } else if (k == "aperture") {
                    if (v == "always") o->aperture_mode = 2;
                    else if (v == "conditional") o->aperture_mode = 1;
                    else if (v == "never") o->aperture_mode = 0;
                    else throw std::invalid_argument(v);
                } else if (k == "aperture_min_length") {
                    o->aperture_min_length = std::stod(v);
                } else if (k == "x_limit") {
                    o->x_limit = std::stod(v);
                } else if (k == "y_limit") {
                    o->y_limit = std::stod(v);
                } else if (k == "stages") {
                    o->stages = std::stoi(v);
                } else if (k == "chunk_words") {
                    o->chunk_words = std::stoi(v);
                } else if (k == "blocks_per_sm") {
                    o->blocks_per_sm = std::stoi(v);
                } else if (k == "track_beambeam4d") {
                    o->track_bb4d = map_flag(v);
                } else if (k == "track_beambeam6d") {
                    o->track_bb6d = map_flag(v);
                } else if (k == "track_spacecharge") {
                    o->track_sc = map_flag(v);
                } else if (k == "track_tricub") {
                    o->track_tricub = map_flag(v);
                } else {
                    if (err) *err = "config: unknown key '" + k + "'";
                    return false;
                }
            } catch (...) {
                if (err) *err = "config: bad value for '" + k + "': '" + v + "'";
                return false;
            }
        }
    }
    // The tracking kernel's block size: track_threads_per_block, else
    // threads_per_block.  The reference accepts up to 1024; this kernel's
    // register budget allows at most kMaxThreads, so larger requests run
    // with kMaxThreads threads per block.
    int const req = o->track_threads_req > 0 ? o->track_threads_req : o->threads_general;
    for (int t : {req, o->threads_general}) {
        if (t < 32 || t > 1024 || t % 32 != 0) {
            if (err) *err = "config: threads_per_block must be a multiple of 32 in [32, 1024]";
            return false;
        }
    }
    o->threads = req < kMaxThreads ? req : kMaxThreads;
    if (o->stages < 2 || o->stages > 8) {
        if (err) *err = "config: stages must be in [2, 8]";
        return false;
    }
    if (o->chunk_words < 64 || o->chunk_words > 8192 || o->chunk_words % 2 != 0) {
        if (err) *err = "config: chunk_words must be even and in [64, 8192]";
        return false;
    }
    return true;
}

// -------------------------------------------------------------- device
struct Device {
    int id = -1;
    cudaStream_t stream = nullptr;
    int32_t *d_flags = nullptr;  // [0] status, [1] error
    int32_t *h_flags = nullptr;  // pinned: [0..1] the flags, [2..3] an int64 count
    // scratch for the active-particle selection (grown on demand, kept)
    uint64_t *scratch = nullptr;
    int64_t scratch_words = 0;
    // recorded after the last work that used `scratch` or `d_flags`
    cudaEvent_t shared_done = nullptr;
};

static std::mutex g_dev_mu;
static std::map<int, Device *> g_devices;
static std::atomic<uint64_t> g_launches{0};

static bool cuda_ok(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

static Device *get_device(int id)
{
    std::lock_guard<std::mutex> lk(g_dev_mu);
    auto it = g_devices.find(id);
    if (it != g_devices.end()) return it->second;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        set_error("no CUDA device available: this engine tracks on the GPU only");
        return nullptr;
    }
    if (id < 0 || id >= count) {
        set_error("device id out of range");
        return nullptr;
    }
    if (!cuda_ok(cudaSetDevice(id), "cudaSetDevice")) return nullptr;
    Device *d = new Device();
    d->id = id;
    if (!cuda_ok(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaMalloc(&d->d_flags, 2 * sizeof(int32_t)), "cudaMalloc") ||
        !cuda_ok(cudaMallocHost(&d->h_flags, 4 * sizeof(int32_t)), "cudaMallocHost") ||
        !cuda_ok(cudaEventCreateWithFlags(&d->shared_done, cudaEventDisableTiming),
                 "cudaEventCreate")) {
        delete d;
        return nullptr;
    }
    g_devices[id] = d;
    return d;
}

// The selection scratch and the status words of a device are shared by
// every call on that device.  Work that uses them is ordered after the
// previous such work on the GPU, also when the two calls launch on different
// streams and return before their kernels finish (the asynchronous entry
// points): the stream first waits for the event the previous user recorded,
// and records it again after its own work.  Inside a stream capture the
// graph orders its own nodes and no event is waited for or recorded.
static bool stream_capturing(cudaStream_t s)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

static bool shared_use_begin(Device *dev, cudaStream_t s)
{
    if (stream_capturing(s)) return true;
    return cuda_ok(cudaStreamWaitEvent(s, dev->shared_done, 0), "cudaStreamWaitEvent");
}

static void shared_use_end(Device *dev, cudaStream_t s)
{
    if (!stream_capturing(s)) cudaEventRecord(dev->shared_done, s);
}

// Brackets one call's use of the shared scratch and status words.
struct SharedUse {
    Device *dev;
    cudaStream_t s;
    bool ok;
    SharedUse(Device *d, cudaStream_t st) : dev(d), s(st), ok(shared_use_begin(d, st)) {}
    ~SharedUse()
    {
        if (ok) shared_use_end(dev, s);
    }
};

// ------------------------------------------------------- device stream
struct DevStream {
    CompiledStream cs;
    uint64_t *d = nullptr;        // chunked stream, the s table, the element offsets
    const double *s_table = nullptr;
    const int64_t *elem_offset = nullptr;
    int device = -1;
    DevStream() = default;
    DevStream(const DevStream &) = delete;
    ~DevStream()
    {
        if (d) cudaFree(d);
    }
};

static std::unique_ptr<DevStream> build_stream(const ImageView &img, uint64_t b, uint64_t e,
                                               const Options &opt, CompileOptions copt,
                                               Device *dev)
{
    std::unique_ptr<DevStream> s(new DevStream());
    copt.aperture_mode = opt.aperture_mode;
    copt.aperture_min_length = opt.aperture_min_length;
    copt.min_chunk_words = opt.chunk_words;
    copt.track_bb4d = opt.track_bb4d;
    copt.track_bb6d = opt.track_bb6d;
    copt.track_sc = opt.track_sc;
    copt.track_tricub = opt.track_tricub;
    std::string err;
    if (!compile_lattice(img, b, e, copt, &s->cs, &err)) {
        set_error(err);
        return nullptr;
    }
    size_t const bytes = s->cs.words.size() * 8;
    size_t const sbytes = s->cs.s_table.size() * 8;
    size_t const obytes = s->cs.elem_offset.size() * 8;
    size_t const side_at = (bytes + sbytes + obytes + 15) & ~(size_t)15;
    size_t const side_bytes = s->cs.side.size() * 8;
    size_t const device_bytes = s->cs.side_device_words * 8;
    if (!cuda_ok(cudaSetDevice(dev->id), "cudaSetDevice") ||
        !cuda_ok(cudaMalloc(&s->d, side_at + side_bytes + device_bytes + 8), "cudaMalloc(lattice)"))
        return nullptr;
    // out-of-line tables: their device addresses go into the records
    uint64_t const side_base = (uint64_t)(uintptr_t)s->d + side_at;
    for (const auto &f : s->cs.side_fixups) s->cs.words[f.first] = side_base + f.second * 8u;
    if ((side_bytes > 0 &&
         !cuda_ok(cudaMemcpy(reinterpret_cast<char *>(s->d) + side_at, s->cs.side.data(),
                             side_bytes, cudaMemcpyHostToDevice),
                  "cudaMemcpy(side tables)")) ||
        !cuda_ok(cudaMemcpy(reinterpret_cast<char *>(s->d) + bytes + sbytes,
                            s->cs.elem_offset.data(), obytes, cudaMemcpyHostToDevice),
                 "cudaMemcpy(element offsets)") ||
        !cuda_ok(cudaMemcpy(s->d, s->cs.words.data(), bytes, cudaMemcpyHostToDevice),
                 "cudaMemcpy(lattice)") ||
        !cuda_ok(cudaMemcpy(reinterpret_cast<char *>(s->d) + bytes, s->cs.s_table.data(), sbytes,
                            cudaMemcpyHostToDevice),
                 "cudaMemcpy(s table)"))
        return nullptr;
    // TriCub cell coefficients, computed on the GPU from the node tables
    if (!s->cs.tricub_tables.empty()) {
        double *side_dev = reinterpret_cast<double *>(reinterpret_cast<char *>(s->d) + side_at);
        for (const auto &t : s->cs.tricub_tables)
            if (!cuda_ok((cudaError_t)launch_tricub_cells(side_dev + t.nodes, side_dev + t.cells,
                                                          t.nx, t.ny, t.nz, nullptr),
                         "tricub cell coefficients"))
                return nullptr;
        if (!cuda_ok(cudaDeviceSynchronize(), "tricub cell coefficients")) return nullptr;
    }
    s->s_table = reinterpret_cast<const double *>(reinterpret_cast<char *>(s->d) + bytes);
    s->elem_offset =
        reinterpret_cast<const int64_t *>(reinterpret_cast<char *>(s->d) + bytes + sbytes);
    s->device = dev->id;
    return s;
}

// Particle-element-turns per launch of a segmented until-turn call: long
// calls are cut into launches of about this much work, and the particles
// still alive are re-packed densely between them (lanes of particles lost
// during a launch stay idle until its end).  ~55 ms of tracking on a GB300.
constexpr double kSegmentPet = 2e9;

static int64_t segment_turns(int64_t active, int64_t num_elements)
{
    double const per_turn = (double)std::max<int64_t>(active, 1) *
                            (double)std::max<int64_t>(num_elements, 1);
    double const t = std::ceil(kSegmentPet / per_turn);
    return t >= 2147483647.0 ? 2147483647 : std::max<int64_t>(1, (int64_t)t);
}

// Run one tracking pass and wait for it; returns the OR-ed status (0/-1).
// An until-turn call that waits is run as a sequence of launches of at most
// segment_turns() turns each, with the particles that still have work
// selected again before every launch; the per-particle arithmetic is the
// same as in one launch, so results are bit-identical.
static int32_t run_track(Device *dev, const Options &opt, const DevStream &ds, uint64_t *d_cols,
                         int64_t n, int64_t i0, int64_t i1, int mode, int64_t until_turn,
                         bool finish_turn, uint64_t *ebe_out, int64_t ebe_cap,
                         const EbeDevConfig *ebe, cudaStream_t stream, bool wait = true)
{
    TrackParams prm{};
    prm.stream = ds.d;
    prm.n_chunks = ds.cs.info.num_chunks;
    prm.chunk_words = ds.cs.info.chunk_words;
    prm.stages = opt.stages;
    prm.mode = mode;
    prm.num_elements = ds.cs.info.num_elements;
    prm.cols = d_cols;
    prm.n = n;
    prm.i0 = i0;
    prm.i1 = i1;
    prm.until_turn = until_turn;
    prm.finish_turn = finish_turn ? 1 : 0;
    prm.xlim_bits = aperture_bits(opt.x_limit);
    prm.ylim_bits = aperture_bits(opt.y_limit);
    prm.status = dev->d_flags;
    prm.error = dev->d_flags + 1;
    prm.ebe_out = ebe_out;
    prm.ebe_cap = ebe_cap;
    prm.s_table = ds.s_table;
    prm.op_mask = ds.cs.info.op_mask;
    if (ebe) prm.ebe = *ebe;
    // stream 0 is the legacy default stream (what torch reports for its
    // default stream): launch there, never substitute another stream
    SharedUse shared(dev, stream);
    if (!shared.ok) return -1;
    if (!cuda_ok(cudaMemsetAsync(dev->d_flags, 0, 2 * sizeof(int32_t), stream), "cudaMemsetAsync"))
        return -1;
    if (i1 > i0 && mode != MODE_EBE) {
        // pack the particles that have work left so warps hold live lanes only
        int64_t const need = select_scratch_words(i1 - i0);
        if (need > dev->scratch_words) {
            if (dev->scratch) cudaFree(dev->scratch);
            dev->scratch = nullptr;
            dev->scratch_words = 0;
            if (!cuda_ok(cudaMalloc(&dev->scratch, (size_t)need * 8), "cudaMalloc(scratch)"))
                return -1;
            dev->scratch_words = need;
        }
        int64_t *idx = nullptr, *count = nullptr;
        int const rs = launch_select(d_cols, n, i0, i1, mode, until_turn, dev->scratch, &idx,
                                     &count, stream);
        if (rs != 0) {
            set_error(std::string("particle selection launch: ") +
                      cudaGetErrorString((cudaError_t)rs));
            return -1;
        }
        g_launches.fetch_add(3);
        prm.idx = idx;
        prm.count = count;
    }
    // until-turn calls that wait: capped launches while work is left (an
    // until_turn within the first segment needs one launch, as the start
    // turns are >= 0 for any particle that can have work)
    int64_t seg = segment_turns(i1 - i0, prm.num_elements);
    bool const segmented = wait && mode == MODE_UNTIL && i1 > i0 && seg < until_turn;
    while (i1 > i0) {
        prm.turn_cap = segmented ? (int32_t)std::min<int64_t>(seg, 2147483647) : 0;
        int const rc = launch_track(prm, opt.fast, opt.threads, opt.blocks_per_sm, stream);
        if (rc != 0) {
            set_error(std::string("track kernel launch: ") + cudaGetErrorString((cudaError_t)rc));
            return -1;
        }
        g_launches.fetch_add(1);
        if (!segmented) break;
        int64_t *idx = nullptr, *count = nullptr;
        int const rs = launch_select(d_cols, n, i0, i1, mode, until_turn, dev->scratch, &idx,
                                     &count, stream);
        if (rs != 0) {
            set_error(std::string("particle selection launch: ") +
                      cudaGetErrorString((cudaError_t)rs));
            return -1;
        }
        g_launches.fetch_add(3);
        int64_t *h_count = reinterpret_cast<int64_t *>(dev->h_flags + 2);
        if (!cuda_ok(cudaMemcpyAsync(h_count, count, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                     stream),
                     "cudaMemcpyAsync(count)") ||
            !cuda_ok(cudaMemcpyAsync(dev->h_flags, dev->d_flags, 2 * sizeof(int32_t),
                                     cudaMemcpyDeviceToHost, stream),
                     "cudaMemcpyAsync(status)") ||
            !cuda_ok(cudaStreamSynchronize(stream), "track kernel"))
            return -1;
        if (*h_count == 0 || dev->h_flags[1] != 0) break;  // done, or a pipeline timeout
        prm.idx = idx;
        prm.count = count;
        seg = segment_turns(*h_count, prm.num_elements);
    }
    if (!wait) return 0;
    if (!cuda_ok(cudaMemcpyAsync(dev->h_flags, dev->d_flags, 2 * sizeof(int32_t),
                                 cudaMemcpyDeviceToHost, stream),
                 "cudaMemcpyAsync(status)") ||
        !cuda_ok(cudaStreamSynchronize(stream), "track kernel"))
        return -1;
    if (dev->h_flags[1] != 0) {
        set_error("track kernel: a shared-memory pipeline wait timed out; the blocks that timed "
                  "out left their particles unchanged, other blocks (and earlier launches of "
                  "the call) may have advanced theirs");
        return -1;
    }
    return dev->h_flags[0];
}

// ------------------------------------------------ particle columns (host)
static double *const *real_cols(const st_Particles *p) { return &p->q0; }
static int64_t *const *int_cols(const st_Particles *p) { return &p->particle_id; }

static void gather(const st_Particles *p, int64_t i0, int64_t cnt, uint64_t *blk)
{
    for (int c = 0; c < 17; ++c) std::memcpy(blk + (size_t)c * cnt, real_cols(p)[c] + i0, cnt * 8);
    for (int c = 0; c < 4; ++c)
        std::memcpy(blk + (size_t)(17 + c) * cnt, int_cols(p)[c] + i0, cnt * 8);
}

static void scatter(st_Particles *p, int64_t i0, int64_t cnt, const uint64_t *blk)
{
    for (int c = 0; c < 17; ++c) std::memcpy(real_cols(p)[c] + i0, blk + (size_t)c * cnt, cnt * 8);
    for (int c = 0; c < 4; ++c)
        std::memcpy(int_cols(p)[c] + i0, blk + (size_t)(17 + c) * cnt, cnt * 8);
}

// Host "generic address" output (NS(ParticlesGenericAddr), particles.h:70-98):
// 1 word count + 21 column addresses.
struct GenericOut {
    const uint64_t *desc = nullptr;
    int64_t n = 0;
    uint64_t *d = nullptr;
    bool download(cudaStream_t s)
    {
        std::vector<uint64_t> blk((size_t)n * 21);
        if (!cuda_ok(cudaMemcpyAsync(blk.data(), d, blk.size() * 8, cudaMemcpyDeviceToHost, s),
                     "cudaMemcpy(output)") ||
            !cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize"))
            return false;
        for (int c = 0; c < 21; ++c)
            std::memcpy((void *)(uintptr_t)desc[1 + c], blk.data() + (size_t)c * n, (size_t)n * 8);
        return true;
    }
    bool upload(cudaStream_t s)
    {
        std::vector<uint64_t> blk((size_t)n * 21);
        for (int c = 0; c < 21; ++c)
            std::memcpy(blk.data() + (size_t)c * n, (const void *)(uintptr_t)desc[1 + c], (size_t)n * 8);
        if (!cuda_ok(cudaMalloc(&d, blk.size() * 8 + 8), "cudaMalloc(output)")) return false;
        return cuda_ok(cudaMemcpyAsync(d, blk.data(), blk.size() * 8, cudaMemcpyHostToDevice, s),
                       "cudaMemcpy(output)") &&
               cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    }
    ~GenericOut()
    {
        if (d) cudaFree(d);
    }
};

// One-shot tracking of host particles (the free functions).
static int32_t track_host(st_Particles *p, int64_t i0, int64_t i1, const st_Buffer *belems,
                          int mode, int64_t until, uint64_t lb, uint64_t le, bool finish,
                          const st_ElemByElemConfig *ebe_cfg)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    if (!p || !belems) {
        set_error("null particles or beam-elements buffer");
        return -1;
    }
    if (i0 < 0 || i1 > p->num_particles || i0 > i1) {
        set_error("particle index out of range");
        return -1;
    }
    Options opt;
    const char *env = std::getenv("SIXTRACKLIB_GB300_CONFIG");
    std::string perr;
    if (env && !parse_options(env, &opt, &perr)) {
        set_error(perr);
        return -1;
    }
    Device *dev = get_device(opt.device);
    if (!dev) return -1;
    cudaSetDevice(dev->id);
    ImageView img;
    std::string err;
    if (!img.open(st_Buffer_get_const_data_begin(belems), st_Buffer_get_size(belems), &err)) {
        set_error(err);
        return -1;
    }
    if (mode == MODE_UNTIL && img.num_objects == 0) return i1 > i0 ? -1 : 0;
    if (mode == MODE_LINE) {
        if (lb > le || le > img.num_objects) {
            set_error("line range outside the lattice");
            return -1;
        }
    }
    cudaStream_t const s = dev->stream;
    std::vector<std::unique_ptr<GenericOut>> outs;
    CompileOptions copt;
    copt.monitor_output = [&](uint64_t ei) -> std::pair<uint64_t, int64_t> {
        const uint64_t *m = img.words(ei);
        if (m[3] == 0) return {0, 0};
        std::unique_ptr<GenericOut> o(new GenericOut());
        o->desc = (const uint64_t *)(uintptr_t)m[3];
        o->n = (int64_t)o->desc[0];
        if (o->n <= 0 || !o->upload(s)) return {0, 0};
        uint64_t const ptr = (uint64_t)(uintptr_t)o->d;
        int64_t const cap = o->n;
        outs.push_back(std::move(o));
        return {ptr, cap};
    };
    uint64_t b = 0, e = img.num_objects;
    if (mode == MODE_LINE) {
        b = lb;
        e = le;
    }
    auto ds = build_stream(img, b, e, opt, copt, dev);
    if (!ds) return -1;
    int64_t const cnt = i1 - i0;
    std::vector<uint64_t> blk((size_t)cnt * 21);
    gather(p, i0, cnt, blk.data());
    uint64_t *d_cols = nullptr;
    GenericOut ebe_out;
    EbeDevConfig ebe{};
    if (mode == MODE_EBE) {
        if (ebe_cfg && ebe_cfg->out_store_addr != 0) {
            ebe_out.desc = (const uint64_t *)(uintptr_t)ebe_cfg->out_store_addr;
            ebe_out.n = (int64_t)ebe_out.desc[0];
            if (!ebe_out.upload(s)) return -1;
            std::memcpy(&ebe, ebe_cfg, sizeof(ebe));
        } else {
            mode = MODE_UNTIL;  // track/track.h:770-775: no output -> until_turn
        }
    }
    int32_t st = -1;
    if (cuda_ok(cudaMalloc(&d_cols, blk.size() * 8 + 8), "cudaMalloc(particles)") &&
        cuda_ok(cudaMemcpyAsync(d_cols, blk.data(), blk.size() * 8, cudaMemcpyHostToDevice, s),
                "cudaMemcpy(particles)")) {
        st = run_track(dev, opt, *ds, d_cols, cnt, 0, cnt, mode, until, finish, ebe_out.d,
                       ebe_out.n, mode == MODE_EBE ? &ebe : nullptr, s);
        bool const ok = cuda_ok(cudaMemcpyAsync(blk.data(), d_cols, blk.size() * 8,
                                                cudaMemcpyDeviceToHost, s),
                                "cudaMemcpy(particles)") &&
                        cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        if (ok) {
            scatter(p, i0, cnt, blk.data());
            for (auto &o : outs) o->download(s);
            if (ebe_out.d) ebe_out.download(s);
        } else {
            st = -1;
        }
    }
    if (d_cols) cudaFree(d_cols);
    return st;
}

}  // namespace stg

using namespace stg;

// =================================================================== C ABI
extern "C" {

st_track_status_t st_Track_particle_until_turn(st_Particles *p, int64_t idx,
                                               const st_Buffer *be, int64_t until_turn)
{
    return track_host(p, idx, idx + 1, be, MODE_UNTIL, until_turn, 0, 0, false, nullptr);
}

st_track_status_t st_Track_all_particles_until_turn(st_Particles *p, const st_Buffer *be,
                                                    int64_t until_turn)
{
    return track_host(p, 0, p ? p->num_particles : 0, be, MODE_UNTIL, until_turn, 0, 0, false,
                      nullptr);
}

st_track_status_t st_Track_particle_element_by_element_until_turn(
    st_Particles *p, int64_t idx, const st_ElemByElemConfig *cfg, const st_Buffer *be,
    int64_t until_turn)
{
    return track_host(p, idx, idx + 1, be, MODE_EBE, until_turn, 0, 0, false, cfg);
}

st_track_status_t st_Track_all_particles_element_by_element_until_turn(
    st_Particles *p, const st_ElemByElemConfig *cfg, const st_Buffer *be, int64_t until_turn)
{
    return track_host(p, 0, p ? p->num_particles : 0, be, MODE_EBE, until_turn, 0, 0, false, cfg);
}

st_track_status_t st_Track_particle_line(st_Particles *p, int64_t idx, const st_Buffer *be,
                                         st_buffer_size_t b, st_buffer_size_t e, bool finish)
{
    return track_host(p, idx, idx + 1, be, MODE_LINE, 0, b, e, finish, nullptr);
}

st_track_status_t st_Track_all_particles_line(st_Particles *p, const st_Buffer *be,
                                              st_buffer_size_t b, st_buffer_size_t e,
                                              bool finish)
{
    return track_host(p, 0, p ? p->num_particles : 0, be, MODE_LINE, 0, b, e, finish, nullptr);
}

uint64_t st_engine_kernel_launches(void) { return g_launches.load(); }

const char *st_engine_build_info(void)
{
    return "sixtracklib_gb300: sm_103a, FP64 tracking kernel (exact | fast), "
           "TMA bulk-copy lattice staging";
}

}  // extern "C"

// ============================================================ DeviceLattice
struct st_DeviceLattice {
    Options opt;
    Device *dev = nullptr;
    std::vector<uint64_t> image;
    std::unique_ptr<DevStream> full;
    std::map<std::pair<uint64_t, uint64_t>, std::unique_ptr<DevStream>> lines;
    cudaStream_t last_stream = nullptr;
};

extern "C" {

st_DeviceLattice *st_DeviceLattice_new(const unsigned char *image, st_buffer_size_t size,
                                       const char *config)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    std::unique_ptr<st_DeviceLattice> L(new st_DeviceLattice());
    std::string err;
    if (!parse_options(config, &L->opt, &err)) {
        set_error(err);
        return nullptr;
    }
    L->dev = get_device(L->opt.device);
    if (!L->dev) return nullptr;
    L->image.assign((size + 7) / 8, 0);
    std::memcpy(L->image.data(), image, size);
    ImageView img;
    if (!img.open(L->image.data(), size, &err)) {
        set_error(err);
        return nullptr;
    }
    L->full = build_stream(img, 0, img.num_objects, L->opt, CompileOptions(), L->dev);
    if (!L->full) return nullptr;
    return L.release();
}

void st_DeviceLattice_delete(st_DeviceLattice *L) { delete L; }

int64_t st_DeviceLattice_num_elements(const st_DeviceLattice *L)
{
    return L ? L->full->cs.info.num_elements : 0;
}
int64_t st_DeviceLattice_num_chunks(const st_DeviceLattice *L)
{
    return L ? L->full->cs.info.num_chunks : 0;
}

st_track_status_t st_DeviceLattice_set_parameters(st_DeviceLattice *L, int64_t num,
                                                  const int64_t *element, const int32_t *kind,
                                                  const double *value)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    if (!L || num < 0 || (num > 0 && (!element || !kind || !value))) {
        set_error("set_parameters: invalid arguments");
        return -1;
    }
    ImageView img;
    std::string err;
    if (!img.open(L->image.data(), L->image.size() * 8, &err)) {
        set_error(err);
        return -1;
    }
    DevStream &ds = *L->full;
    // validate everything before writing anything
    std::vector<std::pair<uint64_t, uint64_t>> where((size_t)num);  // (stream word, image word)
    for (int64_t j = 0; j < num; ++j) {
        int64_t const e = element[j];
        if (e < 0 || e >= ds.cs.info.num_elements) {
            set_error("set_parameters: element index out of range");
            return -1;
        }
        uint64_t const off = (uint64_t)ds.cs.elem_offset[(size_t)e];
        uint64_t const hdr = ds.cs.words[off];
        uint32_t const op = (uint32_t)(hdr & 0xFF);
        uint32_t const order = (uint32_t)(hdr >> 32);
        if (kind[j] >= 0) {
            const uint64_t *bal = img.deref((uint64_t)e, 4);
            if ((op != OP_MULTIPOLE && op != OP_MULTIPOLE_CURV) || !bal ||
                (uint32_t)kind[j] >= 2 * order + 2) {
                set_error("set_parameters: element " + std::to_string(e) +
                          " has no multipole coefficient bal[" + std::to_string(kind[j]) + "]");
                return -1;
            }
            where[(size_t)j] = {off + 1 + (uint64_t)kind[j],
                                (uint64_t)(bal - img.img) + (uint64_t)kind[j]};
        } else if (kind[j] == -1) {
            if (op != OP_CAVITY) {
                set_error("set_parameters: element " + std::to_string(e) + " is not a cavity");
                return -1;
            }
            where[(size_t)j] = {off + 1, img.begin_word((uint64_t)e)};
        } else {
            set_error("set_parameters: unknown parameter kind");
            return -1;
        }
    }
    if (!cuda_ok(cudaSetDevice(L->dev->id), "cudaSetDevice") ||
        !cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize"))
        return -1;
    for (int64_t j = 0; j < num; ++j) {
        uint64_t bits;
        std::memcpy(&bits, &value[j], 8);
        ds.cs.words[where[(size_t)j].first] = bits;
        L->image[where[(size_t)j].second] = bits;
    }
    if (!cuda_ok(cudaMemcpy(ds.d, ds.cs.words.data(), ds.cs.words.size() * 8,
                            cudaMemcpyHostToDevice),
                 "cudaMemcpy(lattice)"))
        return -1;
    L->lines.clear();  // line streams are rebuilt from the updated image
    return 0;
}

st_track_status_t st_DeviceLattice_track_until(st_DeviceLattice *L, void *d_cols, int64_t n,
                                               int64_t until_turn, void *stream)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    if (L && n == 0) return 0;
    if (!L || !d_cols) return -1;
    if (L->full->cs.info.num_elements == 0) {  // track/track.h:617: an empty lattice fails
        set_error("st_DeviceLattice_track_until: empty lattice");
        return -1;
    }
    cudaSetDevice(L->dev->id);
    return run_track(L->dev, L->opt, *L->full, (uint64_t *)d_cols, n, 0, n, MODE_UNTIL,
                     until_turn, false, nullptr, 0, nullptr, (cudaStream_t)stream);
}

st_track_status_t st_DeviceLattice_track_line(st_DeviceLattice *L, void *d_cols, int64_t n,
                                              uint64_t b, uint64_t e, bool finish, void *stream)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    if (L && n == 0) return 0;
    if (!L || !d_cols) return -1;
    auto key = std::make_pair(b, e);
    auto it = L->lines.find(key);
    if (it == L->lines.end()) {
        ImageView img;
        std::string err;
        img.open(L->image.data(), L->image.size() * 8, &err);
        auto ds = build_stream(img, b, e, L->opt, CompileOptions(), L->dev);
        if (!ds) return -1;
        it = L->lines.emplace(key, std::move(ds)).first;
    }
    cudaSetDevice(L->dev->id);
    return run_track(L->dev, L->opt, *it->second, (uint64_t *)d_cols, n, 0, n, MODE_LINE, 0,
                     finish, nullptr, 0, nullptr, (cudaStream_t)stream);
}

int32_t st_DeviceLattice_launch_until(st_DeviceLattice *L, void *d_cols, int64_t n,
                                      int64_t until_turn, void *stream)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    if (L && n == 0) return 0;
    if (!L || !d_cols) return -1;
    if (L->full->cs.info.num_elements == 0) {  // track/track.h:617: an empty lattice fails
        set_error("st_DeviceLattice_launch_until: empty lattice");
        return -1;
    }
    cudaSetDevice(L->dev->id);
    L->last_stream = (cudaStream_t)stream;
    return run_track(L->dev, L->opt, *L->full, (uint64_t *)d_cols, n, 0, n, MODE_UNTIL,
                     until_turn, false, nullptr, 0, nullptr, L->last_stream, false);
}

st_track_status_t st_DeviceLattice_last_status(st_DeviceLattice *L)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    if (!L) return -1;
    cudaStream_t s = L->last_stream;
    if (!shared_use_begin(L->dev, s)) return -1;
    if (!cuda_ok(cudaMemcpyAsync(L->dev->h_flags, L->dev->d_flags, 2 * sizeof(int32_t),
                                 cudaMemcpyDeviceToHost, s),
                 "cudaMemcpyAsync(status)") ||
        !cuda_ok(cudaStreamSynchronize(s), "track kernel"))
        return -1;
    if (L->dev->h_flags[1] != 0) {
        set_error("track kernel: shared-memory pipeline wait timed out");
        return -1;
    }
    return L->dev->h_flags[0];
}

}  // extern "C"

// ================================================================ TrackJob
struct OutBlock {
    uint64_t obj_index = 0;  // Particles object in the output buffer
    int64_t cap = 0;
    uint64_t *d = nullptr;   // device column block (inside the job's output arena)
};

struct st_TrackJob {
    Options opt;
    std::string arch = "cuda", config, device_id_str;
    Device *dev = nullptr;
    st_Buffer *pbuf = nullptr, *ebuf = nullptr, *obuf = nullptr;
    bool owns_obuf = false;
    std::vector<st_buffer_size_t> psets;
    std::vector<int64_t> pset_off, pset_cnt;
    int64_t n_total = 0;
    uint64_t *d_cols = nullptr;
    std::unique_ptr<DevStream> lat;
    std::map<std::pair<uint64_t, uint64_t>, std::unique_ptr<DevStream>> lines;
    uint64_t *d_out = nullptr;
    std::vector<OutBlock> outs;  // [ebe?] + monitors
    bool has_ebe = false;
    st_ElemByElemConfig ebe_cfg{};
    uint64_t ebe_out_offset = 0, bemon_out_offset = 0;
    uint64_t until_turn_ebe = 0;
    std::vector<st_buffer_size_t> monitor_indices;
    std::map<uint64_t, size_t> monitor_block;  // element index -> outs index
    int64_t min_pid = 0, max_pid = 0, min_elem = 0, max_elem = 0, min_turn = 0, max_turn = 0;
    uint16_t collect_flags = 0x05;  // particles | output (track/definitions.h)
    bool default_rolling = true;
    // the particle buffer's memory, page-locked for direct DMA (or null)
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
    // device column addresses of the particle sets (fetch_particle_addresses)
    std::vector<st_ParticlesAddr> paddr;
    std::vector<bool> paddr_set;
    // debug mode (track/track_job_base.h:182-189): inputs validated before
    // every tracking call, the outcome kept in a debug register
    bool debug_mode = false;
    uint64_t debug_reg = 0;
    // stored buffers (id -> buffer, owned) and assignment items; kept
    // across reset, freed with the job
    std::map<uint64_t, std::pair<st_Buffer *, bool>> stored;
    uint64_t next_stored_id = 1024;
    std::deque<st_AssignAddressItem> assign_items;

    ~st_TrackJob()
    {
        release();
        for (auto &kv : stored)
            if (kv.second.second && kv.second.first) st_Buffer_delete(kv.second.first);
        stored.clear();
    }
    void release()
    {
        if (pinned) cudaHostUnregister(pinned);
        pinned = nullptr;
        pinned_bytes = 0;
        paddr.clear();
        paddr_set.clear();
        if (d_cols) cudaFree(d_cols);
        if (d_out) cudaFree(d_out);
        d_cols = nullptr;
        d_out = nullptr;
        lat.reset();
        lines.clear();
        outs.clear();
        if (owns_obuf && obuf) st_Buffer_delete(obuf);
        obuf = nullptr;
        owns_obuf = false;
        monitor_block.clear();
        monitor_indices.clear();
        has_ebe = false;
    }
};

namespace {

st_Particles *pset(st_TrackJob *j, size_t k)
{
    return st_Particles_buffer_get_particles(j->pbuf, j->psets[k]);
}

// Page-lock the caller's particle buffer for the job's lifetime so that
// push / collect are direct DMA copies of the columns (no staging copy on
// the host).  The buffer is caller-owned and outlives the job (the
// reference's ownership rule); when it cannot be registered (already
// registered by another job, or unsupported) the staged copy is used.
void pin_particles(st_TrackJob *j)
{
    unsigned char *base = st_Buffer_get_data_begin(j->pbuf);
    size_t const bytes = (size_t)st_Buffer_get_capacity(j->pbuf);
    if (!base || bytes == 0) return;
    if (cudaHostRegister(base, bytes, cudaHostRegisterDefault) == cudaSuccess) {
        j->pinned = base;
        j->pinned_bytes = bytes;
    } else {
        (void)cudaGetLastError();  // not fatal: staged copies
    }
}

// Column c of particle set k (host pointer) when the whole column lies in
// the page-locked range, else null.
void *pinned_column(st_TrackJob *j, size_t k, int c)
{
    if (!j->pinned || st_Buffer_get_data_begin(j->pbuf) != j->pinned) return nullptr;
    st_Particles *p = pset(j, k);
    void *col = c < 17 ? (void *)real_cols(p)[c] : (void *)int_cols(p)[c - 17];
    uintptr_t const a = (uintptr_t)col, b = (uintptr_t)j->pinned;
    size_t const bytes = (size_t)j->pset_cnt[k] * 8;
    if (a < b || a + bytes > b + j->pinned_bytes) return nullptr;
    return col;
}

// Direct column copies between the page-locked buffer and the device block.
bool copy_pinned(st_TrackJob *j, bool to_device)
{
    if (!j->pinned) return false;
    for (size_t k = 0; k < j->psets.size(); ++k)
        for (int c = 0; c < 21; ++c)
            if (!pinned_column(j, k, c)) return false;
    cudaStream_t s = j->dev->stream;
    for (size_t k = 0; k < j->psets.size(); ++k) {
        size_t const bytes = (size_t)j->pset_cnt[k] * 8;
        if (bytes == 0) continue;
        for (int c = 0; c < 21; ++c) {
            uint64_t *dcol = j->d_cols + (size_t)c * j->n_total + j->pset_off[k];
            void *hcol = pinned_column(j, k, c);
            cudaError_t const e =
                to_device ? cudaMemcpyAsync(dcol, hcol, bytes, cudaMemcpyHostToDevice, s)
                          : cudaMemcpyAsync(hcol, dcol, bytes, cudaMemcpyDeviceToHost, s);
            if (!cuda_ok(e, "cudaMemcpyAsync(particles)")) return false;
        }
    }
    return cuda_ok(cudaStreamSynchronize(s), "particle copy");
}

bool upload_particles(st_TrackJob *j)
{
    if (j->pinned && copy_pinned(j, true)) return true;
    std::vector<uint64_t> blk((size_t)j->n_total * 21);
    for (size_t k = 0; k < j->psets.size(); ++k) {
        st_Particles *p = pset(j, k);
        int64_t const cnt = j->pset_cnt[k];
        std::vector<uint64_t> part((size_t)cnt * 21);
        gather(p, 0, cnt, part.data());
        for (int c = 0; c < 21; ++c)
            std::memcpy(blk.data() + (size_t)c * j->n_total + j->pset_off[k],
                        part.data() + (size_t)c * cnt, (size_t)cnt * 8);
    }
    return cuda_ok(cudaMemcpy(j->d_cols, blk.data(), blk.size() * 8, cudaMemcpyHostToDevice),
                   "cudaMemcpy(particles)");
}

bool download_particles(st_TrackJob *j)
{
    if (j->pinned && copy_pinned(j, false)) return true;
    std::vector<uint64_t> blk((size_t)j->n_total * 21);
    if (!cuda_ok(cudaMemcpy(blk.data(), j->d_cols, blk.size() * 8, cudaMemcpyDeviceToHost),
                 "cudaMemcpy(particles)"))
        return false;
    for (size_t k = 0; k < j->psets.size(); ++k) {
        int64_t const cnt = j->pset_cnt[k];
        std::vector<uint64_t> part((size_t)cnt * 21);
        for (int c = 0; c < 21; ++c)
            std::memcpy(part.data() + (size_t)c * cnt,
                        blk.data() + (size_t)c * j->n_total + j->pset_off[k], (size_t)cnt * 8);
        scatter(pset(j, k), 0, cnt, part.data());
    }
    return true;
}

bool transfer_outputs(st_TrackJob *j, bool to_device)
{
    for (const OutBlock &o : j->outs) {
        st_Particles *p = st_Particles_buffer_get_particles(j->obuf, o.obj_index);
        if (!p) return false;
        std::vector<uint64_t> blk((size_t)o.cap * 21);
        if (to_device) {
            gather(p, 0, o.cap, blk.data());
            if (!cuda_ok(cudaMemcpy(o.d, blk.data(), blk.size() * 8, cudaMemcpyHostToDevice),
                         "cudaMemcpy(output)"))
                return false;
        } else {
            if (!cuda_ok(cudaMemcpy(blk.data(), o.d, blk.size() * 8, cudaMemcpyDeviceToHost),
                         "cudaMemcpy(output)"))
                return false;
            scatter(p, 0, o.cap, blk.data());
        }
    }
    return true;
}

bool compile_job_lattice(st_TrackJob *j)
{
    ImageView img;
    std::string err;
    if (!img.open(st_Buffer_get_const_data_begin(j->ebuf), st_Buffer_get_size(j->ebuf), &err)) {
        set_error(err);
        return false;
    }
    CompileOptions copt;
    copt.monitor_output = [j](uint64_t ei) -> std::pair<uint64_t, int64_t> {
        auto it = j->monitor_block.find(ei);
        if (it == j->monitor_block.end()) return {0, 0};
        const OutBlock &o = j->outs[it->second];
        return {(uint64_t)(uintptr_t)o.d, o.cap};
    };
    j->lat = build_stream(img, 0, img.num_objects, j->opt, copt, j->dev);
    j->lines.clear();
    return j->lat != nullptr;
}

// Min/max attributes (output/output_buffer.h:461-560,
// elem_by_elem_output_buffer.h:162-230) and output preparation
// (output/output_buffer.c:288-360, be_monitor/output_buffer.c).
bool setup_job(st_TrackJob *j, st_Buffer *pb, st_buffer_size_t nsets, const st_buffer_size_t *idx,
               st_Buffer *eb, st_Buffer *ob, st_buffer_size_t until_ebe)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    j->release();
    if (!pb || !eb) {
        set_error("TrackJob: particles and beam-elements buffers are required");
        return false;
    }
    j->pbuf = pb;
    j->ebuf = eb;
    j->psets.clear();
    if (nsets > 0 && idx) {
        j->psets.assign(idx, idx + nsets);
    } else {
        for (st_buffer_size_t i = 0; i < st_Buffer_get_num_of_objects(pb); ++i)
            if (st_Particles_buffer_get_particles(pb, i)) {
                j->psets.push_back(i);
                break;
            }
    }
    if (j->psets.empty()) {
        set_error("TrackJob: no particle set in the particles buffer");
        return false;
    }
    j->pset_off.clear();
    j->pset_cnt.clear();
    j->n_total = 0;
    bool first = true;
    for (size_t k = 0; k < j->psets.size(); ++k) {
        st_Particles *p = pset(j, k);
        if (!p) {
            set_error("TrackJob: particle set index does not name a Particles object");
            return false;
        }
        j->pset_off.push_back(j->n_total);
        j->pset_cnt.push_back(p->num_particles);
        j->n_total += p->num_particles;
        for (int64_t i = 0; i < p->num_particles; ++i) {
            int64_t const pid = p->particle_id[i], ae = p->at_element_id[i], at = p->at_turn[i];
            if (first) {
                j->min_pid = j->max_pid = pid;
                j->min_elem = j->max_elem = ae;
                j->min_turn = j->max_turn = at;
                first = false;
            }
            j->min_pid = std::min(j->min_pid, pid);
            j->max_pid = std::max(j->max_pid, pid);
            j->min_elem = std::min(j->min_elem, ae);
            j->max_elem = std::max(j->max_elem, ae);
            j->min_turn = std::min(j->min_turn, at);
            j->max_turn = std::max(j->max_turn, at);
        }
    }
    if (j->min_pid < 0) j->min_pid = 0;
    if (j->min_elem < 0) j->min_elem = 0;
    if (j->min_turn < 0) j->min_turn = 0;
    // element id range of the lattice (every object counts as an element)
    uint64_t const ne = st_Buffer_get_num_of_objects(eb);
    if (ne > 0) {
        j->min_elem = std::min<int64_t>(j->min_elem, 0);
        j->max_elem = std::max<int64_t>(j->max_elem, (int64_t)ne - 1);
    }
    // beam monitors that get output
    std::vector<uint64_t> mons;
    const st_Object *ob_begin = st_Buffer_get_const_objects_begin(eb);
    for (uint64_t i = 0; i < ne; ++i) {
        if (ob_begin[i].type_id != ST_OBJECT_TYPE_BEAM_MONITOR) continue;
        j->monitor_indices.push_back(i);
        st_BeamMonitor *m = (st_BeamMonitor *)(uintptr_t)ob_begin[i].begin_addr;
        if (m->start >= j->min_turn && m->num_stores > 0) mons.push_back(i);
    }
    j->until_turn_ebe = 0;
    bool const want_ebe = until_ebe > 0 && until_ebe > (uint64_t)j->min_turn;
    if (want_ebe || !mons.empty()) {
        if (!ob) {
            ob = st_Buffer_new(0);
            if (!ob) return false;
            j->owns_obuf = true;
        }
        j->obuf = ob;
    } else {
        j->obuf = ob;
    }
    std::vector<std::pair<uint64_t, int64_t>> blocks;  // (obj index, cap)
    if (want_ebe) {
        st_ElemByElemConfig_init_detailed(&j->ebe_cfg, 0, j->min_pid, j->max_pid, j->min_elem,
                                          j->max_elem, j->min_turn, (int64_t)until_ebe - 1,
                                          j->default_rolling);
        int64_t const cap = st_ElemByElemConfig_get_stored_num_particles(&j->ebe_cfg);
        j->ebe_out_offset = st_Buffer_get_num_of_objects(j->obuf);
        if (!st_Particles_new(j->obuf, (st_buffer_size_t)cap)) return false;
        blocks.push_back({j->ebe_out_offset, cap});
        j->has_ebe = true;
        j->until_turn_ebe = until_ebe;
    }
    j->bemon_out_offset = j->obuf ? st_Buffer_get_num_of_objects(j->obuf) : 0;
    for (uint64_t i : mons) {
        st_BeamMonitor *m = (st_BeamMonitor *)(uintptr_t)st_Buffer_get_const_objects_begin(eb)[i].begin_addr;
        m->min_particle_id = j->min_pid;
        m->max_particle_id = j->max_pid;
        m->out_address = 0;
        int64_t const cap = (j->max_pid - j->min_pid + 1) * m->num_stores;
        uint64_t const oi = st_Buffer_get_num_of_objects(j->obuf);
        if (!st_Particles_new(j->obuf, (st_buffer_size_t)cap)) return false;
        j->monitor_block[i] = blocks.size();
        blocks.push_back({oi, cap});
    }
    // device allocations
    cudaSetDevice(j->dev->id);
    if (!cuda_ok(cudaMalloc(&j->d_cols, (size_t)std::max<int64_t>(j->n_total, 1) * 21 * 8),
                 "cudaMalloc(particles)"))
        return false;
    size_t total = 0;
    for (auto &b : blocks) total += (size_t)b.second * 21;
    if (total > 0 && !cuda_ok(cudaMalloc(&j->d_out, total * 8), "cudaMalloc(output)")) return false;
    size_t off = 0;
    for (auto &b : blocks) {
        OutBlock o;
        o.obj_index = b.first;
        o.cap = b.second;
        o.d = j->d_out + off;
        off += (size_t)b.second * 21;
        j->outs.push_back(o);
    }
    pin_particles(j);
    if (!upload_particles(j) || !transfer_outputs(j, true)) return false;
    return compile_job_lattice(j);
}

bool arch_ok(const char *arch)
{
    std::string a = arch ? arch : "cuda";
    std::transform(a.begin(), a.end(), a.begin(), ::tolower);
    a = trim(a);
    if (a.empty() || a == "cuda" || a == "gb300" || a == "gpu") return true;
    set_error("TrackJob: architecture '" + a +
              "' is not provided by this engine (it tracks on the GPU: use \"cuda\")");
    return false;
}

st_TrackJob *make_job(const char *arch, const char *cfg)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    if (!arch_ok(arch)) return nullptr;
    std::unique_ptr<st_TrackJob> j(new st_TrackJob());
    std::string err;
    if (!parse_options(cfg, &j->opt, &err)) {
        set_error(err);
        return nullptr;
    }
    j->config = cfg ? cfg : "";
    j->dev = get_device(j->opt.device);
    if (!j->dev) return nullptr;
    j->device_id_str = "0." + std::to_string(j->dev->id);
    return j.release();
}

}  // namespace

extern "C" {

st_TrackJob *st_TrackJob_create(const char *arch, const char *cfg) { return make_job(arch, cfg); }

st_TrackJob *st_TrackJob_new(const char *arch, st_Buffer *pb, st_Buffer *eb, const char *cfg)
{
    return st_TrackJob_new_detailed(arch, pb, 0, nullptr, eb, nullptr, 0, cfg);
}

st_TrackJob *st_TrackJob_new_with_output(const char *arch, st_Buffer *pb, st_Buffer *eb,
                                         st_Buffer *ob, st_buffer_size_t until_ebe,
                                         const char *cfg)
{
    return st_TrackJob_new_detailed(arch, pb, 0, nullptr, eb, ob, until_ebe, cfg);
}

st_TrackJob *st_TrackJob_new_detailed(const char *arch, st_Buffer *pb, st_buffer_size_t nsets,
                                      const st_buffer_size_t *idx, st_Buffer *eb,
                                      st_Buffer *ob, st_buffer_size_t until_ebe, const char *cfg)
{
    st_TrackJob *j = make_job(arch, cfg);
    if (!j) return nullptr;
    if (!setup_job(j, pb, nsets, idx, eb, ob, until_ebe)) {
        std::string const e = st_last_error();
        delete j;
        set_error(e);
        return nullptr;
    }
    return j;
}

bool st_TrackJob_reset(st_TrackJob *j, st_Buffer *pb, st_Buffer *eb, st_Buffer *ob)
{
    return j && setup_job(j, pb, 0, nullptr, eb, ob, 0);
}
bool st_TrackJob_reset_with_output(st_TrackJob *j, st_Buffer *pb, st_Buffer *eb, st_Buffer *ob,
                                   st_buffer_size_t until_ebe)
{
    return j && setup_job(j, pb, 0, nullptr, eb, ob, until_ebe);
}
bool st_TrackJob_reset_detailed(st_TrackJob *j, st_Buffer *pb, st_buffer_size_t nsets,
                                const st_buffer_size_t *idx, st_Buffer *eb, st_Buffer *ob,
                                st_buffer_size_t until_ebe)
{
    return j && setup_job(j, pb, nsets, idx, eb, ob, until_ebe);
}

void st_TrackJob_delete(st_TrackJob *j) { delete j; }
void st_TrackJob_clear(st_TrackJob *j)
{
    if (j) j->release();
}

}  // extern "C"

// Debug register of a job in debug mode (the reference's CUDA debug
// kernels, track/track_kernel_impl.h:149-250): input flags from
// SIXTRL_ARCH_DEBUGGING_MIN_FLAG = 2^32 up (control/definitions.h:105-117),
// the track status in the low 32 bits (control/debug_register.h:59-80).
constexpr uint64_t kDbgParticleIdxIllegal = 1ull << 32;
constexpr uint64_t kDbgPbufferNull = 1ull << 33;
constexpr uint64_t kDbgBelemBufferNull = 1ull << 34;
constexpr uint64_t kDbgPsetIndexIllegal = 1ull << 36;
constexpr uint64_t kDbgPbufferRemap = 1ull << 37;
constexpr uint64_t kDbgBelemBufferRemap = 1ull << 38;
constexpr uint64_t kDbgLineBoundariesIllegal = 1ull << 39;
constexpr uint64_t kDbgUntilTurnIllegal = 1ull << 40;
// the engine's own flags, above the reference's
constexpr uint64_t kDbgPipelineTimeout = 1ull << 41;
constexpr uint64_t kDbgNoElemByElemOutput = 1ull << 42;

static uint64_t debug_input_flags(const st_TrackJob *j, int64_t until_turn, bool line,
                                  uint64_t b, uint64_t e)
{
    uint64_t f = 0;
    if (!j->pbuf) f |= kDbgPbufferNull;
    if (!j->ebuf) f |= kDbgBelemBufferNull;
    if (j->pbuf && st_Buffer_needs_remapping(j->pbuf)) f |= kDbgPbufferRemap;
    if (j->ebuf && st_Buffer_needs_remapping(j->ebuf)) f |= kDbgBelemBufferRemap;
    if (j->pbuf)
        for (st_buffer_size_t k : j->psets)
            if (k >= st_Buffer_get_num_of_objects(j->pbuf) ||
                !st_Particles_buffer_get_const_particles(j->pbuf, k))
                f |= kDbgPsetIndexIllegal;
    if (j->n_total < 0) f |= kDbgParticleIdxIllegal;
    if (until_turn < 0) f |= kDbgUntilTurnIllegal;
    if (line && (b > e || !j->ebuf || e > st_Buffer_get_num_of_objects(j->ebuf)))
        f |= kDbgLineBoundariesIllegal;
    return f;
}

// Runs `track` unless the inputs fail validation, and records the outcome;
// returns the reference's status: the track status, or failure when any
// flag is raised.
template <class F>
static st_track_status_t debug_track(st_TrackJob *j, uint64_t flags, F track)
{
    int32_t status = -1;
    if (flags == 0) {
        status = track();
        if (j->dev && j->dev->h_flags[1] != 0) flags |= kDbgPipelineTimeout;
    }
    j->debug_reg = flags | (uint64_t)(uint32_t)status;
    return flags != 0 ? -1 : status;
}

extern "C" {

st_track_status_t st_TrackJob_track_until(st_TrackJob *j, st_buffer_size_t until_turn)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    if (!j || !j->lat) return -1;
    clear_error();
    auto track = [&]() -> int32_t {
        cudaSetDevice(j->dev->id);
        if (j->lat->cs.info.num_elements == 0) return j->n_total > 0 ? -1 : 0;
        return run_track(j->dev, j->opt, *j->lat, j->d_cols, j->n_total, 0, j->n_total,
                         MODE_UNTIL, (int64_t)until_turn, false, nullptr, 0, nullptr,
                         j->dev->stream);
    };
    if (j->debug_mode)
        return debug_track(j, debug_input_flags(j, (int64_t)until_turn, false, 0, 0), track);
    return track();
}

st_track_status_t st_TrackJob_track_elem_by_elem(st_TrackJob *j, st_buffer_size_t until_turn)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    if (!j || !j->lat) return -1;
    clear_error();
    if (j->debug_mode) {
        uint64_t f = debug_input_flags(j, (int64_t)until_turn, false, 0, 0);
        if (!j->has_ebe || j->outs.empty()) f |= kDbgNoElemByElemOutput;
        if (f != 0) return debug_track(j, f, [] { return -1; });
        j->debug_mode = false;  // validated: run the plain call, then record it
        st_track_status_t const st = st_TrackJob_track_elem_by_elem(j, until_turn);
        j->debug_mode = true;
        return debug_track(j, 0, [st] { return st; });
    }
    if (!j->has_ebe || j->outs.empty()) {
        set_error("TrackJob: no elem-by-elem output configured (until_turn_elem_by_elem)");
        return -1;
    }
    cudaSetDevice(j->dev->id);
    EbeDevConfig ebe;
    std::memcpy(&ebe, &j->ebe_cfg, sizeof(ebe));
    const OutBlock &o = j->outs[0];
    return run_track(j->dev, j->opt, *j->lat, j->d_cols, j->n_total, 0, j->n_total, MODE_EBE,
                     (int64_t)until_turn, false, o.d, o.cap, &ebe, j->dev->stream);
}

st_track_status_t st_TrackJob_track_line(st_TrackJob *j, st_buffer_size_t b, st_buffer_size_t e,
                                         bool finish)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    if (!j || !j->lat) return -1;
    clear_error();
    if (j->debug_mode) {
        uint64_t const f = debug_input_flags(j, 0, true, b, e);
        if (f != 0) return debug_track(j, f, [] { return -1; });
        j->debug_mode = false;
        st_track_status_t const st = st_TrackJob_track_line(j, b, e, finish);
        j->debug_mode = true;
        return debug_track(j, 0, [st] { return st; });
    }
    uint64_t const ne = st_Buffer_get_num_of_objects(j->ebuf);
    if (b > e || e > ne) {
        set_error("TrackJob: line range outside the lattice");
        return -1;
    }
    auto key = std::make_pair((uint64_t)b, (uint64_t)e);
    auto it = j->lines.find(key);
    if (it == j->lines.end()) {
        ImageView img;
        std::string err;
        if (!img.open(st_Buffer_get_const_data_begin(j->ebuf), st_Buffer_get_size(j->ebuf), &err)) {
            set_error(err);
            return -1;
        }
        CompileOptions copt;
        copt.monitor_output = [j](uint64_t ei) -> std::pair<uint64_t, int64_t> {
            auto mit = j->monitor_block.find(ei);
            if (mit == j->monitor_block.end()) return {0, 0};
            const OutBlock &o = j->outs[mit->second];
            return {(uint64_t)(uintptr_t)o.d, o.cap};
        };
        auto ds = build_stream(img, b, e, j->opt, copt, j->dev);
        if (!ds) return -1;
        it = j->lines.emplace(key, std::move(ds)).first;
    }
    cudaSetDevice(j->dev->id);
    return run_track(j->dev, j->opt, *it->second, j->d_cols, j->n_total, 0, j->n_total, MODE_LINE,
                     0, finish, nullptr, 0, nullptr, j->dev->stream);
}

void st_TrackJob_collect_particles(st_TrackJob *j)
{
    if (j && j->d_cols) download_particles(j);
}
void st_TrackJob_collect_beam_elements(st_TrackJob *j) { (void)j; }
void st_TrackJob_collect_output(st_TrackJob *j)
{
    if (j && !j->outs.empty()) transfer_outputs(j, false);
}
void st_TrackJob_collect_detailed(st_TrackJob *j, uint16_t flags)
{
    if (!j) return;
    if (flags & 0x01) st_TrackJob_collect_particles(j);
    if (flags & 0x02) st_TrackJob_collect_beam_elements(j);
    if (flags & 0x04) st_TrackJob_collect_output(j);
}
void st_TrackJob_collect(st_TrackJob *j)
{
    if (j) st_TrackJob_collect_detailed(j, j->collect_flags);
}
void st_TrackJob_push_particles(st_TrackJob *j)
{
    if (j && j->d_cols) upload_particles(j);
}
void st_TrackJob_push_beam_elements(st_TrackJob *j)
{
    if (j && j->ebuf) compile_job_lattice(j);
}
void st_TrackJob_push_output(st_TrackJob *j)
{
    if (j && !j->outs.empty()) transfer_outputs(j, true);
}
void st_TrackJob_push(st_TrackJob *j, uint16_t flags)
{
    if (!j) return;
    if (flags & 0x01) st_TrackJob_push_particles(j);
    if (flags & 0x02) st_TrackJob_push_beam_elements(j);
    if (flags & 0x04) st_TrackJob_push_output(j);
}

void st_TrackJob_enable_collect_particles(st_TrackJob *j) { if (j) j->collect_flags |= 0x01; }
void st_TrackJob_disable_collect_particles(st_TrackJob *j) { if (j) j->collect_flags &= ~0x01; }
bool st_TrackJob_is_collecting_particles(const st_TrackJob *j) { return j && (j->collect_flags & 0x01); }
void st_TrackJob_enable_collect_beam_elements(st_TrackJob *j) { if (j) j->collect_flags |= 0x02; }
void st_TrackJob_disable_collect_beam_elements(st_TrackJob *j) { if (j) j->collect_flags &= ~0x02; }
bool st_TrackJob_is_collecting_beam_elements(const st_TrackJob *j) { return j && (j->collect_flags & 0x02); }
void st_TrackJob_enable_collect_output(st_TrackJob *j) { if (j) j->collect_flags |= 0x04; }
void st_TrackJob_disable_collect_output(st_TrackJob *j) { if (j) j->collect_flags &= ~0x04; }
bool st_TrackJob_is_collecting_output(const st_TrackJob *j) { return j && (j->collect_flags & 0x04); }
uint16_t st_TrackJob_get_collect_flags(const st_TrackJob *j) { return j ? j->collect_flags : 0; }
void st_TrackJob_set_collect_flags(st_TrackJob *j, uint16_t f) { if (j) j->collect_flags = f; }
bool st_TrackJob_requires_collecting(const st_TrackJob *j) { return j != nullptr; }

// SIXTRL_ARCHITECTURE_CUDA (control/definitions.h:84-86): the id a CUDA
// track job reports (cuda/track/track_job.cpp:129)
int64_t st_TrackJob_get_type_id(const st_TrackJob *j) { return j ? 3 : -1; }
uint32_t st_TrackJobNew_get_arch_id(const st_TrackJobBaseNew *j) { return j ? 3u : 0u; }
bool st_TrackJobNew_has_arch_string(const st_TrackJobBaseNew *j) { return j != nullptr; }
st_buffer_size_t st_CudaTrackJob_get_num_available_nodes(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return (st_buffer_size_t)n;
}
st_buffer_size_t st_CudaTrackJob_get_available_node_indices_list(st_buffer_size_t max_num,
                                                                 int64_t *indices)
{
    st_buffer_size_t const n = st_CudaTrackJob_get_num_available_nodes();
    st_buffer_size_t k = 0;
    for (; indices && k < n && k < max_num; ++k) indices[k] = (int64_t)k;
    return k;
}
const char *st_TrackJob_get_type_str(const st_TrackJob *j) { return j ? "cuda" : ""; }
bool st_TrackJob_has_device_id_str(const st_TrackJob *j) { return j && !j->device_id_str.empty(); }
const char *st_TrackJob_get_device_id_str(const st_TrackJob *j)
{
    return j ? j->device_id_str.c_str() : "";
}
bool st_TrackJob_has_config_str(const st_TrackJob *j) { return j && !j->config.empty(); }
const char *st_TrackJob_get_config_str(const st_TrackJob *j) { return j ? j->config.c_str() : ""; }
st_buffer_size_t st_TrackJob_get_num_particle_sets(const st_TrackJob *j)
{
    return j ? j->psets.size() : 0;
}
const st_buffer_size_t *st_TrackJob_get_particle_set_indices_begin(const st_TrackJob *j)
{
    return (j && !j->psets.empty()) ? j->psets.data() : nullptr;
}
const st_buffer_size_t *st_TrackJob_get_particle_set_indices_end(const st_TrackJob *j)
{
    return (j && !j->psets.empty()) ? j->psets.data() + j->psets.size() : nullptr;
}
st_buffer_size_t st_TrackJob_get_particle_set_index(const st_TrackJob *j, st_buffer_size_t n)
{
    return (j && n < j->psets.size()) ? j->psets[n] : (st_buffer_size_t)-1;
}
st_buffer_size_t st_TrackJob_get_total_num_particles_in_sets(const st_TrackJob *j)
{
    return j ? (st_buffer_size_t)j->n_total : 0;
}
int64_t st_TrackJob_get_min_particle_id(const st_TrackJob *j) { return j ? j->min_pid : -1; }
int64_t st_TrackJob_get_max_particle_id(const st_TrackJob *j) { return j ? j->max_pid : -1; }
int64_t st_TrackJob_get_min_element_id(const st_TrackJob *j) { return j ? j->min_elem : -1; }
int64_t st_TrackJob_get_max_element_id(const st_TrackJob *j) { return j ? j->max_elem : -1; }
int64_t st_TrackJob_get_min_initial_turn_id(const st_TrackJob *j) { return j ? j->min_turn : -1; }
int64_t st_TrackJob_get_max_initial_turn_id(const st_TrackJob *j) { return j ? j->max_turn : -1; }
st_Buffer *st_TrackJob_get_particles_buffer(st_TrackJob *j) { return j ? j->pbuf : nullptr; }
const st_Buffer *st_TrackJob_get_const_particles_buffer(const st_TrackJob *j)
{
    return j ? j->pbuf : nullptr;
}
st_Buffer *st_TrackJob_get_beam_elements_buffer(st_TrackJob *j) { return j ? j->ebuf : nullptr; }
const st_Buffer *st_TrackJob_get_const_beam_elements_buffer(const st_TrackJob *j)
{
    return j ? j->ebuf : nullptr;
}
bool st_TrackJob_has_output_buffer(const st_TrackJob *j) { return j && j->obuf; }
bool st_TrackJob_owns_output_buffer(const st_TrackJob *j) { return j && j->owns_obuf; }
st_Buffer *st_TrackJob_get_output_buffer(st_TrackJob *j) { return j ? j->obuf : nullptr; }
const st_Buffer *st_TrackJob_get_const_output_buffer(const st_TrackJob *j)
{
    return j ? j->obuf : nullptr;
}
bool st_TrackJob_has_elem_by_elem_output(const st_TrackJob *j) { return j && j->has_ebe; }
bool st_TrackJob_has_beam_monitor_output(const st_TrackJob *j)
{
    return j && !j->monitor_block.empty();
}
st_buffer_size_t st_TrackJob_get_elem_by_elem_output_buffer_offset(const st_TrackJob *j)
{
    return j ? j->ebe_out_offset : 0;
}
st_buffer_size_t st_TrackJob_get_beam_monitor_output_buffer_offset(const st_TrackJob *j)
{
    return j ? j->bemon_out_offset : 0;
}
st_buffer_size_t st_TrackJob_get_num_elem_by_elem_turns(const st_TrackJob *j)
{
    return j ? j->until_turn_ebe : 0;
}
bool st_TrackJob_has_elem_by_elem_config(const st_TrackJob *j) { return j && j->has_ebe; }
const st_ElemByElemConfig *st_TrackJob_get_elem_by_elem_config(const st_TrackJob *j)
{
    return (j && j->has_ebe) ? &j->ebe_cfg : nullptr;
}
bool st_TrackJob_is_elem_by_elem_config_rolling(const st_TrackJob *j)
{
    return j && j->has_ebe && j->ebe_cfg.is_rolling != 0;
}
bool st_TrackJob_get_default_elem_by_elem_config_rolling_flag(const st_TrackJob *j)
{
    return j && j->default_rolling;
}
void st_TrackJob_set_default_elem_by_elem_config_rolling_flag(st_TrackJob *j, bool r)
{
    if (j) j->default_rolling = r;
}
int64_t st_TrackJob_get_elem_by_elem_config_order(const st_TrackJob *j)
{
    return (j && j->has_ebe) ? j->ebe_cfg.order : -1;
}
bool st_TrackJob_has_beam_monitors(const st_TrackJob *j) { return j && !j->monitor_indices.empty(); }
st_buffer_size_t st_TrackJob_get_num_beam_monitors(const st_TrackJob *j)
{
    return j ? j->monitor_indices.size() : 0;
}
const st_buffer_size_t *st_TrackJob_get_beam_monitor_indices_begin(const st_TrackJob *j)
{
    return (j && !j->monitor_indices.empty()) ? j->monitor_indices.data() : nullptr;
}
const st_buffer_size_t *st_TrackJob_get_beam_monitor_indices_end(const st_TrackJob *j)
{
    return (j && !j->monitor_indices.empty())
               ? j->monitor_indices.data() + j->monitor_indices.size()
               : nullptr;
}
st_buffer_size_t st_TrackJob_get_beam_monitor_index(const st_TrackJob *j, st_buffer_size_t n)
{
    return (j && n < j->monitor_indices.size()) ? j->monitor_indices[n] : (st_buffer_size_t)-1;
}

// ----------------------------------------------- TrackJobNew / CudaTrackJob
st_CudaTrackJob *st_CudaTrackJob_create(void) { return make_job("cuda", nullptr); }
st_CudaTrackJob *st_CudaTrackJob_new_from_config_str(const char *cfg) { return make_job("cuda", cfg); }
st_CudaTrackJob *st_CudaTrackJob_new(const char *node_id, st_Buffer *pb, st_Buffer *eb)
{
    return st_CudaTrackJob_new_detailed(node_id, pb, 0, nullptr, eb, nullptr, 0, nullptr);
}
st_CudaTrackJob *st_CudaTrackJob_new_with_output(const char *node_id, st_Buffer *pb,
                                                 st_Buffer *eb, st_Buffer *ob,
                                                 st_buffer_size_t until_ebe)
{
    return st_CudaTrackJob_new_detailed(node_id, pb, 0, nullptr, eb, ob, until_ebe, nullptr);
}
st_CudaTrackJob *st_CudaTrackJob_new_detailed(const char *node_id, st_Buffer *pb,
                                              st_buffer_size_t nsets,
                                              const st_buffer_size_t *idx, st_Buffer *eb,
                                              st_Buffer *ob, st_buffer_size_t until_ebe,
                                              const char *cfg)
{
    // node id "platform.device" (cuda/track_job.h:42-66): the device index
    // is the part after the dot.
    std::string c = cfg ? cfg : "";
    if (node_id && *node_id) {
        std::string nid(node_id);
        size_t const dot = nid.find('.');
        std::string const dev = (dot == std::string::npos) ? nid : nid.substr(dot + 1);
        if (!dev.empty() && std::all_of(dev.begin(), dev.end(), ::isdigit))
            c += (c.empty() ? "" : "\n") + std::string("device=") + dev;
    }
    return st_TrackJob_new_detailed("cuda", pb, nsets, idx, eb, ob, until_ebe, c.c_str());
}
void st_TrackJobNew_delete(st_TrackJobBaseNew *j) { delete j; }
st_track_status_t st_TrackJobNew_track_until(st_TrackJobBaseNew *j, st_buffer_size_t u)
{
    return st_TrackJob_track_until(j, u);
}
bool st_TrackJobNew_is_in_debug_mode(const st_TrackJobBaseNew *j) { return j && j->debug_mode; }
int32_t st_TrackJobNew_enable_debug_mode(st_TrackJobBaseNew *j)
{
    if (!j) return -1;
    j->debug_mode = true;
    j->debug_reg = 0;
    return 0;
}
int32_t st_TrackJobNew_disable_debug_mode(st_TrackJobBaseNew *j)
{
    if (!j) return -1;
    j->debug_mode = false;
    return 0;
}
int32_t st_TrackJobNew_collect_debug_flag(st_TrackJobBaseNew *j)
{
    // the register is written on the host by every call in debug mode
    return (j && j->debug_mode) ? 0 : -1;
}
uint64_t st_TrackJobNew_get_debug_register(const st_TrackJobBaseNew *j)
{
    return j ? j->debug_reg : 0;
}
st_track_status_t st_TrackJobNew_track_elem_by_elem(st_TrackJobBaseNew *j, st_buffer_size_t u)
{
    return st_TrackJob_track_elem_by_elem(j, u);
}
st_track_status_t st_TrackJobNew_track_line(st_TrackJobBaseNew *j, st_buffer_size_t b,
                                            st_buffer_size_t e, bool f)
{
    return st_TrackJob_track_line(j, b, e, f);
}
int32_t st_TrackJobNew_collect_particles(st_TrackJobBaseNew *j)
{
    return (j && download_particles(j)) ? 0 : -1;
}
int32_t st_TrackJobNew_collect_beam_elements(st_TrackJobBaseNew *j) { return j ? 0 : -1; }
int32_t st_TrackJobNew_collect_output(st_TrackJobBaseNew *j)
{
    return (j && transfer_outputs(j, false)) ? 0 : -1;
}
int32_t st_TrackJobNew_collect(st_TrackJobBaseNew *j)
{
    if (!j) return -1;
    st_TrackJob_collect(j);
    return 0;
}
int32_t st_TrackJobNew_push_particles(st_TrackJobBaseNew *j)
{
    return (j && upload_particles(j)) ? 0 : -1;
}
int32_t st_TrackJobNew_push_beam_elements(st_TrackJobBaseNew *j)
{
    return (j && compile_job_lattice(j)) ? 0 : -1;
}
int32_t st_TrackJobNew_push_output(st_TrackJobBaseNew *j)
{
    return (j && transfer_outputs(j, true)) ? 0 : -1;
}
// ------------------------------------------ stored buffers, address items
// Without ownership the job keeps the caller's pointer.  With ownership the
// contents move into a buffer of the job's (object addresses unchanged), the
// caller's buffer is left empty and is deleted if delete_ptr_after_move
// (track_job_buffer_store.cpp:255-283).
st_buffer_size_t st_TrackJob_add_stored_buffer(st_TrackJob *j, st_Buffer *b, bool own,
                                               bool delete_ptr_after_move)
{
    if (!j || !b) return 0;
    st_Buffer *kept = b;
    if (own) {
        kept = buffer_take_contents(b);
        if (!kept) return 0;
        if (delete_ptr_after_move) st_Buffer_delete(b);
    }
    uint64_t const id = j->next_stored_id++;
    j->stored[id] = {kept, own};
    return id;
}
st_buffer_size_t st_TrackJob_create_stored_buffer(st_TrackJob *j, st_buffer_size_t cap)
{
    if (!j) return 0;
    st_Buffer *b = st_Buffer_new(cap);
    if (!b) return 0;
    uint64_t const id = j->next_stored_id++;
    j->stored[id] = {b, true};
    return id;
}
int32_t st_TrackJob_remove_stored_buffer(st_TrackJob *j, st_buffer_size_t id)
{
    if (!j) return -1;
    auto it = j->stored.find(id);
    if (it == j->stored.end()) return -1;
    if (it->second.second && it->second.first) st_Buffer_delete(it->second.first);
    j->stored.erase(it);
    return 0;
}
bool st_TrackJob_has_stored_buffers(const st_TrackJob *j) { return j && !j->stored.empty(); }
st_buffer_size_t st_TrackJob_num_stored_buffers(const st_TrackJob *j)
{
    return j ? j->stored.size() : 0;
}
st_buffer_size_t st_TrackJob_min_stored_buffer_id(const st_TrackJob *j)
{
    return (j && !j->stored.empty()) ? j->stored.begin()->first : 0;
}
st_buffer_size_t st_TrackJob_max_stored_buffer_id(const st_TrackJob *j)
{
    return (j && !j->stored.empty()) ? j->stored.rbegin()->first : 0;
}
bool st_TrackJob_owns_stored_buffer(const st_TrackJob *j, st_buffer_size_t id)
{
    if (!j) return false;
    auto it = j->stored.find(id);
    return it != j->stored.end() && it->second.second;
}
st_Buffer *st_TrackJob_stored_buffer(st_TrackJob *j, st_buffer_size_t id)
{
    if (!j) return nullptr;
    auto it = j->stored.find(id);
    return it != j->stored.end() ? it->second.first : nullptr;
}
const st_Buffer *st_TrackJob_const_stored_buffer(const st_TrackJob *j, st_buffer_size_t id)
{
    return st_TrackJob_stored_buffer(const_cast<st_TrackJob *>(j), id);
}

static bool same_item(const st_AssignAddressItem &a, const st_AssignAddressItem &b)
{
    return std::memcmp(&a, &b, sizeof(a)) == 0;
}
static bool pair_of(const st_AssignAddressItem &a, uint64_t dest, uint64_t src)
{
    return a.dest_buffer_id == dest && a.src_buffer_id == src;
}
// The st_Buffer a buffer id names: 1 particles, 2 beam elements, 3 output,
// >= 1024 stored.
static st_Buffer *buffer_of(st_TrackJob *j, uint64_t id)
{
    if (id == 1) return j->pbuf;
    if (id == 2) return j->ebuf;
    if (id == 3) return j->obuf;
    auto it = j->stored.find(id);
    return it != j->stored.end() ? it->second.first : nullptr;
}
// Address of (object `index`, byte `off`) of buffer `b` if the object has
// the type `tid` and holds 8 bytes at `off`; 0 otherwise
// (buffer/assign_address_item.h: *_from_managed_buffer).
static uint64_t field_addr(st_Buffer *b, uint64_t index, uint64_t tid, uint64_t off)
{
    if (!b || index >= st_Buffer_get_num_of_objects(b)) return 0;
    const st_Object &o = st_Buffer_get_const_objects_begin(b)[index];
    uint64_t const a = o.begin_addr + off;
    if (o.begin_addr == 0 || o.type_id != tid || o.size < off + 8 || a % 8 != 0) return 0;
    return a;
}

st_AssignAddressItem *st_TrackJob_add_assign_address_item(st_TrackJob *j,
                                                          const st_AssignAddressItem *item)
{
    if (!j || !item) return nullptr;
    for (auto &it : j->assign_items)
        if (same_item(it, *item)) return &it;
    j->assign_items.push_back(*item);
    return &j->assign_items.back();
}
st_AssignAddressItem *st_TrackJob_add_assign_address_item_detailed(
    st_TrackJob *j, st_object_type_id_t dt, st_buffer_size_t db, st_buffer_size_t di,
    st_buffer_size_t doff, st_object_type_id_t stid, st_buffer_size_t sb, st_buffer_size_t si,
    st_buffer_size_t soff)
{
    st_AssignAddressItem const it{db, sb, dt, stid, di, si, doff, soff};
    return st_TrackJob_add_assign_address_item(j, &it);
}
const st_AssignAddressItem *st_TrackJob_ptr_assign_address_item(const st_TrackJob *j,
                                                                 const st_AssignAddressItem *item)
{
    if (!j || !item) return nullptr;
    for (auto const &it : j->assign_items)
        if (same_item(it, *item)) return &it;
    return nullptr;
}
bool st_TrackJob_has_assign_address_item(const st_TrackJob *j, const st_AssignAddressItem *item)
{
    return st_TrackJob_ptr_assign_address_item(j, item) != nullptr;
}
st_buffer_size_t st_TrackJob_num_assign_items(const st_TrackJob *j, st_buffer_size_t dest,
                                              st_buffer_size_t src)
{
    if (!j) return 0;
    st_buffer_size_t n = 0;
    for (auto const &it : j->assign_items) n += pair_of(it, dest, src) ? 1 : 0;
    return n;
}
bool st_TrackJob_has_assign_items(const st_TrackJob *j, st_buffer_size_t dest,
                                  st_buffer_size_t src)
{
    return st_TrackJob_num_assign_items(j, dest, src) > 0;
}
st_buffer_size_t st_TrackJob_total_num_assign_items(const st_TrackJob *j)
{
    return j ? j->assign_items.size() : 0;
}
const st_AssignAddressItem *st_TrackJob_ptr_assign_address_item_by_index(
    const st_TrackJob *j, st_buffer_size_t dest, st_buffer_size_t src, st_buffer_size_t index)
{
    if (!j) return nullptr;
    st_buffer_size_t k = 0;
    for (auto const &it : j->assign_items)
        if (pair_of(it, dest, src) && k++ == index) return &it;
    return nullptr;
}
bool st_TrackJob_has_assign_item_by_index(const st_TrackJob *j, st_buffer_size_t dest,
                                          st_buffer_size_t src, st_buffer_size_t index)
{
    return st_TrackJob_ptr_assign_address_item_by_index(j, dest, src, index) != nullptr;
}
// Index among the items of the item's (dest, src) pair; that pair's count
// when the item is not there.
st_buffer_size_t st_TrackJob_index_of_assign_address_item(const st_TrackJob *j,
                                                          const st_AssignAddressItem *item)
{
    if (!j || !item) return 0;
    st_buffer_size_t k = 0;
    for (auto const &it : j->assign_items) {
        if (!pair_of(it, item->dest_buffer_id, item->src_buffer_id)) continue;
        if (same_item(it, *item)) return k;
        ++k;
    }
    return k;
}
int32_t st_TrackJob_commit_address_assignments(st_TrackJob *j)
{
    if (!j) return -1;
    clear_error();
    for (auto const &it : j->assign_items) {
        st_Buffer *d = buffer_of(j, it.dest_buffer_id), *s = buffer_of(j, it.src_buffer_id);
        if (!d || !s || it.dest_elem_index >= st_Buffer_get_num_of_objects(d) ||
            it.src_elem_index >= st_Buffer_get_num_of_objects(s)) {
            set_error("TrackJob: an assignment item names a missing buffer or object");
            return -1;
        }
    }
    return 0;
}
static int32_t assign(st_TrackJob *j, bool all, uint64_t dest, uint64_t src)
{
    if (!j) return -1;
    clear_error();
    bool lattice = false;
    for (auto const &it : j->assign_items) {
        if (!all && !pair_of(it, dest, src)) continue;
        uint64_t const sa = field_addr(buffer_of(j, it.src_buffer_id), it.src_elem_index,
                                       it.src_elem_type_id, it.src_pointer_offset);
        uint64_t const da = field_addr(buffer_of(j, it.dest_buffer_id), it.dest_elem_index,
                                       it.dest_elem_type_id, it.dest_pointer_offset);
        if (!sa || !da || it.dest_buffer_id == 1) {
            set_error("TrackJob: an assignment item does not match its objects");
            return -1;
        }
        *(uint64_t *)(uintptr_t)da = sa;
        lattice = lattice || it.dest_buffer_id == 2;
    }
    if (lattice && !compile_job_lattice(j)) return -1;
    return 0;
}
int32_t st_TrackJob_assign_all_addresses(st_TrackJob *j) { return assign(j, true, 0, 0); }
int32_t st_TrackJob_assign_addresses(st_TrackJob *j, st_buffer_size_t dest, st_buffer_size_t src)
{
    return assign(j, false, dest, src);
}
// The engine reads stored buffers from host memory when it compiles the
// lattice: a push recompiles when an item reads this buffer.
int32_t st_TrackJob_push_stored_buffer(st_TrackJob *j, st_buffer_size_t id)
{
    if (!j || !st_TrackJob_stored_buffer(j, id)) return -1;
    for (auto const &it : j->assign_items)
        if (it.src_buffer_id == id && it.dest_buffer_id == 2)
            return compile_job_lattice(j) ? 0 : -1;
    return 0;
}
// The engine writes a stored buffer only through BeamMonitors whose
// out_address was assigned from it: the monitor's turn-by-turn records (the
// job's own monitor output, in the reference's layout) are copied into the
// assigned particle set, as many particles as both hold.
int32_t st_TrackJob_collect_stored_buffer(st_TrackJob *j, st_buffer_size_t id)
{
    st_Buffer *sb = j ? st_TrackJob_stored_buffer(j, id) : nullptr;
    if (!sb) return -1;
    bool collected = false;
    for (auto const &it : j->assign_items) {
        if (it.src_buffer_id != id || it.dest_buffer_id != 2 ||
            it.dest_elem_type_id != ST_OBJECT_TYPE_BEAM_MONITOR)
            continue;
        auto mb = j->monitor_block.find(it.dest_elem_index);
        if (mb == j->monitor_block.end()) continue;
        if (!collected) {
            st_TrackJob_collect_output(j);
            collected = true;
        }
        const st_Particles *src =
            st_Particles_buffer_get_particles(j->obuf, j->outs[mb->second].obj_index);
        st_Particles *dst = st_Particles_buffer_get_particles(sb, it.src_elem_index);
        if (!src || !dst) continue;
        int64_t const n = std::min(src->num_particles, dst->num_particles);
        std::vector<uint64_t> blk((size_t)n * 21);
        gather(src, 0, n, blk.data());
        scatter(dst, 0, n, blk.data());
    }
    return 0;
}

bool st_TrackJob_can_fetch_particles_addr(const st_TrackJob *j) { return j && j->d_cols; }
bool st_TrackJob_has_particles_addr(const st_TrackJob *j)
{
    if (!j) return false;
    for (bool b : j->paddr_set)
        if (b) return true;
    return false;
}
// The device block holds column c of all tracked particles contiguously:
// set k's column c starts at d_cols + c * n_total + pset_off[k].
int32_t st_TrackJob_fetch_particle_addresses(st_TrackJob *j)
{
    if (!j || !j->d_cols) return -1;
    j->paddr.assign(j->psets.size(), st_ParticlesAddr{});
    j->paddr_set.assign(j->psets.size(), true);
    for (size_t k = 0; k < j->psets.size(); ++k) {
        st_ParticlesAddr &a = j->paddr[k];
        a.num_particles = j->pset_cnt[k];
        uint64_t *cols = &a.q0_addr;
        for (int c = 0; c < 21; ++c)
            cols[c] = (uint64_t)(uintptr_t)(j->d_cols + (size_t)c * j->n_total + j->pset_off[k]);
    }
    return 0;
}
static int pset_position(const st_TrackJob *j, st_buffer_size_t index)
{
    for (size_t k = 0; k < j->psets.size(); ++k)
        if (j->psets[k] == index) return (int)k;
    return -1;
}
int32_t st_TrackJob_clear_particle_addresses(st_TrackJob *j, st_buffer_size_t index)
{
    if (!j) return -1;
    int const k = pset_position(j, index);
    if (k < 0 || (size_t)k >= j->paddr_set.size()) return -1;
    j->paddr_set[k] = false;
    return 0;
}
int32_t st_TrackJob_clear_all_particle_addresses(st_TrackJob *j)
{
    if (!j) return -1;
    j->paddr.clear();
    j->paddr_set.clear();
    return 0;
}
const st_ParticlesAddr *st_TrackJob_particle_addresses(const st_TrackJob *j,
                                                        st_buffer_size_t index)
{
    if (!j) return nullptr;
    int const k = pset_position(j, index);
    if (k < 0 || (size_t)k >= j->paddr_set.size() || !j->paddr_set[k]) return nullptr;
    return &j->paddr[k];
}
bool st_TrackJobNew_can_fetch_particle_addresses(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_can_fetch_particles_addr(j);
}
bool st_TrackJobNew_has_particle_addresses(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_has_particles_addr(j);
}
int32_t st_TrackJobNew_fetch_particle_addresses(st_TrackJobBaseNew *j)
{
    return st_TrackJob_fetch_particle_addresses(j);
}
int32_t st_TrackJobNew_clear_particle_addresses(st_TrackJobBaseNew *j, st_buffer_size_t i)
{
    return st_TrackJob_clear_particle_addresses(j, i);
}
int32_t st_TrackJobNew_clear_all_particle_addresses(st_TrackJobBaseNew *j)
{
    return st_TrackJob_clear_all_particle_addresses(j);
}
const st_ParticlesAddr *st_TrackJobNew_get_particle_addresses(const st_TrackJobBaseNew *j,
                                                               st_buffer_size_t i)
{
    return st_TrackJob_particle_addresses(j, i);
}
st_TrackJobBaseNew *st_TrackJobNew_create(const char *arch, const char *cfg)
{
    return st_TrackJob_create(arch, cfg);
}
st_TrackJobBaseNew *st_TrackJobNew_new(const char *arch, st_Buffer *pb, st_Buffer *eb,
                                       const char *cfg)
{
    return st_TrackJob_new_detailed(arch, pb, 0, nullptr, eb, nullptr, 0, cfg);
}
st_TrackJobBaseNew *st_TrackJobNew_new_with_output(const char *arch, st_Buffer *pb, st_Buffer *eb,
                                                   st_Buffer *ob, st_buffer_size_t until_ebe,
                                                   const char *cfg)
{
    return st_TrackJob_new_detailed(arch, pb, 0, nullptr, eb, ob, until_ebe, cfg);
}
st_TrackJobBaseNew *st_TrackJobNew_new_detailed(const char *arch, st_Buffer *pb,
                                                st_buffer_size_t nsets,
                                                const st_buffer_size_t *idx, st_Buffer *eb,
                                                st_Buffer *ob, st_buffer_size_t until_ebe,
                                                const char *cfg)
{
    return st_TrackJob_new_detailed(arch, pb, nsets, idx, eb, ob, until_ebe, cfg);
}
int32_t st_TrackJobNew_reset(st_TrackJobBaseNew *j, st_Buffer *pb, st_Buffer *eb, st_Buffer *ob)
{
    return st_TrackJob_reset(j, pb, eb, ob) ? 0 : -1;
}
int32_t st_TrackJobNew_reset_with_output(st_TrackJobBaseNew *j, st_Buffer *pb, st_Buffer *eb,
                                         st_Buffer *ob, st_buffer_size_t until_ebe)
{
    return st_TrackJob_reset_with_output(j, pb, eb, ob, until_ebe) ? 0 : -1;
}
int32_t st_TrackJobNew_reset_detailed(st_TrackJobBaseNew *j, st_Buffer *pb,
                                      st_buffer_size_t nsets, const st_buffer_size_t *idx,
                                      st_Buffer *eb, st_Buffer *ob, st_buffer_size_t until_ebe)
{
    return st_TrackJob_reset_detailed(j, pb, nsets, idx, eb, ob, until_ebe) ? 0 : -1;
}
void st_TrackJobNew_clear(st_TrackJobBaseNew *j) { st_TrackJob_clear(j); }
uint16_t st_TrackJobNew_push(st_TrackJobBaseNew *j, uint16_t flags)
{
    if (!j) return 0;
    st_TrackJob_push(j, flags);
    return (uint16_t)(flags & 0x07);
}
bool st_TrackJobNew_requires_collecting(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_requires_collecting(j);
}
st_Buffer *st_TrackJobNew_get_particles_buffer(st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_particles_buffer(j);
}
const st_Buffer *st_TrackJobNew_get_const_particles_buffer(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_const_particles_buffer(j);
}
st_Buffer *st_TrackJobNew_get_beam_elements_buffer(st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_beam_elements_buffer(j);
}
const st_Buffer *st_TrackJobNew_get_const_beam_elements_buffer(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_const_beam_elements_buffer(j);
}
bool st_TrackJobNew_has_output_buffer(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_has_output_buffer(j);
}
bool st_TrackJobNew_owns_output_buffer(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_owns_output_buffer(j);
}
st_Buffer *st_TrackJobNew_get_output_buffer(st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_output_buffer(j);
}
const st_Buffer *st_TrackJobNew_get_const_output_buffer(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_const_output_buffer(j);
}
bool st_TrackJobNew_has_elem_by_elem_output(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_has_elem_by_elem_output(j);
}
bool st_TrackJobNew_has_beam_monitor_output(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_has_beam_monitor_output(j);
}
st_buffer_size_t st_TrackJobNew_get_elem_by_elem_output_buffer_offset(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_elem_by_elem_output_buffer_offset(j);
}
st_buffer_size_t st_TrackJobNew_get_beam_monitor_output_buffer_offset(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_beam_monitor_output_buffer_offset(j);
}
st_buffer_size_t st_TrackJobNew_get_num_beam_monitors(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_num_beam_monitors(j);
}
bool st_TrackJobNew_has_beam_monitors(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_has_beam_monitors(j);
}
st_buffer_size_t st_TrackJobNew_get_num_particle_sets(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_num_particle_sets(j);
}
st_buffer_size_t st_TrackJobNew_get_total_num_of_particles(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_total_num_particles_in_sets(j);
}
const char *st_TrackJobNew_get_arch_string(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_type_str(j);
}
bool st_TrackJobNew_has_config_str(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_has_config_str(j);
}
const char *st_TrackJobNew_get_config_str(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_config_str(j);
}
uint16_t st_TrackJobNew_get_collect_flags(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_get_collect_flags(j);
}
void st_TrackJobNew_set_collect_flags(st_TrackJobBaseNew *j, uint16_t f)
{
    st_TrackJob_set_collect_flags(j, f);
}
bool st_TrackJobNew_is_collecting_particles(const st_TrackJobBaseNew *j)
{
    return st_TrackJob_is_collecting_particles(j);
}
void st_TrackJobNew_enable_collect_particles(st_TrackJobBaseNew *j)
{
    st_TrackJob_enable_collect_particles(j);
}
void st_TrackJobNew_disable_collect_particles(st_TrackJobBaseNew *j)
{
    st_TrackJob_disable_collect_particles(j);
}
uint64_t st_CudaTrackJob_default_track_threads_per_block(const st_CudaTrackJob *j)
{
    return j ? (uint64_t)j->opt.threads : 0;
}
uint64_t st_CudaTrackJob_default_threads_per_block(const st_CudaTrackJob *j)
{
    return j ? (uint64_t)j->opt.threads_general : 0;
}

}  // extern "C"

// ------------------------------------------- launch view (for noalloc.cu)
#include "lattice_view.h"

namespace stg {

bool device_lattice_view(const st_DeviceLattice *L, LatticeLaunchView *v)
{
    if (!L || !L->full || !L->dev || !v) return false;
    v->stream = L->full->d;
    v->s_table = L->full->s_table;
    v->n_chunks = L->full->cs.info.num_chunks;
    v->chunk_words = L->full->cs.info.chunk_words;
    v->stages = L->opt.stages;
    v->threads = L->opt.threads;
    v->blocks_per_sm = L->opt.blocks_per_sm;
    v->num_elements = L->full->cs.info.num_elements;
    v->fast = L->opt.fast;
    v->xlim_bits = aperture_bits(L->opt.x_limit);
    v->ylim_bits = aperture_bits(L->opt.y_limit);
    v->device = L->dev->id;
    v->elem_offset = L->full->elem_offset;
    v->op_mask = L->full->cs.info.op_mask;
    return true;
}

// Selection scratch of `device`, grown to at least `words` (engine-owned).
uint64_t *device_scratch(int device, int64_t words)
{
    Device *dev = get_device(device);
    if (!dev) return nullptr;
    if (words > dev->scratch_words) {
        if (dev->scratch) cudaFree(dev->scratch);
        dev->scratch = nullptr;
        dev->scratch_words = 0;
        if (!cuda_ok(cudaMalloc(&dev->scratch, (size_t)words * 8), "cudaMalloc(scratch)"))
            return nullptr;
        dev->scratch_words = words;
    }
    return dev->scratch;
}

bool shared_scratch_begin(int device, void *stream)
{
    Device *dev = get_device(device);
    return dev && shared_use_begin(dev, static_cast<cudaStream_t>(stream));
}

void shared_scratch_end(int device, void *stream)
{
    Device *dev = get_device(device);
    if (dev) shared_use_end(dev, static_cast<cudaStream_t>(stream));
}

void count_launches(uint64_t n) { g_launches.fetch_add(n); }

}  // namespace stg

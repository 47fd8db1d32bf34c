// batch.cu -- many lattice variants tracked by one persistent kernel.
//
// A batch holds V compiled lattices (st_DeviceLattice) and, for each, a
// device-resident particle column block.  One launch of the persistent
// batch kernel advances every variant by `turns_per_launch` turns: the work
// is cut into tiles of threads_per_block particles of one variant, ordered
// longest lattice first, and the CTAs (as many as fit on the GPU) take
// tiles from a global counter until none is left.  Small variants therefore
// share the GPU with large ones instead of each occupying it alone, as
// per-lattice launches do.
//
// A run of launches can be captured into a CUDA graph; the graph reads the
// turn it starts from in device memory and advances it, so the same graph
// replays turn after turn.  The launch shape (threads per block, register
// tier, shared-memory stages, turns per launch) is chosen by an autotuner
// that times candidate shapes on a sample of the batch's own particles.
//
// The arithmetic is the tracking kernel's (the same device function, same
// arithmetic policy): a particle's result is bit-identical to tracking its
// lattice alone with st_DeviceLattice_track_until.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "common.h"
#include "device_guard.h"
#include "kernel_api.h"
#include "lattice_view.h"

namespace stg {
namespace {

__global__ void set_turn_kernel(int64_t *base, int64_t value) { *base = value; }
__global__ void add_turn_kernel(int64_t *base, int64_t delta) { *base += delta; }

bool cuda_ok(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

struct Shape {
    int threads = 128;
    int blocks_per_sm = 2;
    int stages = 4;
    int turns_per_launch = 1;
};

bool parse_shape(const char *cfg, Shape *sh, std::string *err)
{
    if (!cfg) return true;
    std::string s(cfg);
    for (char &c : s)
        if (c == ';' || c == ',' || c == '\n') c = ' ';
    std::istringstream in(s);
    std::string tok;
    while (in >> tok) {
        size_t const eq = tok.find('=');
        if (eq == std::string::npos) {
            *err = "batch config: expected key=value, got '" + tok + "'";
            return false;
        }
        std::string const k = tok.substr(0, eq), v = tok.substr(eq + 1);
        int val = 0;
        try {
            val = std::stoi(v);
        } catch (...) {
            *err = "batch config: bad value for '" + k + "'";
            return false;
        }
        if (k == "threads_per_block" || k == "threads") sh->threads = val;
        else if (k == "blocks_per_sm") sh->blocks_per_sm = val;
        else if (k == "stages") sh->stages = val;
        else if (k == "turns_per_launch") sh->turns_per_launch = val;
        else {
            *err = "batch config: unknown key '" + k + "'";
            return false;
        }
    }
    return true;
}

bool shape_valid(const Shape &sh, std::string *err)
{
    if (sh.threads < 32 || sh.threads > kMaxThreads || sh.threads % 32 != 0) {
        *err = "batch config: threads_per_block must be a multiple of 32 in [32, 256]";
        return false;
    }
    if (sh.stages < 2 || sh.stages > 8) {
        *err = "batch config: stages must be in [2, 8]";
        return false;
    }
    if (sh.blocks_per_sm < 1 || sh.blocks_per_sm > 2) {
        *err = "batch config: blocks_per_sm must be 1 or 2";
        return false;
    }
    if (sh.turns_per_launch < 1) {
        *err = "batch config: turns_per_launch must be >= 1";
        return false;
    }
    return true;
}

// Device-side launch tables for one shape and one set of particle blocks.
struct Plan {
    Shape shape;
    TrackParams *d_variants = nullptr;
    BatchItem *d_items = nullptr;
    int32_t num_items = 0;
    unsigned grid = 0;
    size_t smem = 0;
    bool plain = false;  // every variant is a plain ring: the plain-ring kernel
    void release()
    {
        if (d_variants) cudaFree(d_variants);
        if (d_items) cudaFree(d_items);
        d_variants = nullptr;
        d_items = nullptr;
        num_items = 0;
    }
};

}  // namespace
}  // namespace stg

using namespace stg;

struct st_BatchTracker {
    int device = 0;
    bool fast = false;
    int sm_count = 0;
    std::vector<LatticeLaunchView> views;
    std::vector<uint64_t *> cols;
    std::vector<int64_t> n;
    Plan plan;
    cudaStream_t stream = nullptr;  // own stream (capturable)
    int64_t *d_base = nullptr;      // turn the next launch sequence starts from
    int32_t *d_flags = nullptr;     // status, error
    int32_t *h_flags = nullptr;     // pinned
    int32_t *d_counters = nullptr;
    int64_t n_counters = 0;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    int64_t graph_turns = 0;
    ~st_BatchTracker()
    {
        if (device >= 0) cudaSetDevice(device);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        plan.release();
        if (d_base) cudaFree(d_base);
        if (d_flags) cudaFree(d_flags);
        if (h_flags) cudaFreeHost(h_flags);
        if (d_counters) cudaFree(d_counters);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int max_chunk_words(const st_BatchTracker *b)
{
    int cw = 64;
    for (const auto &v : b->views) cw = std::max(cw, (int)v.chunk_words);
    return cw;
}

// Build the launch tables of `sh` for particle blocks `cols` / `n`.
bool build_plan(st_BatchTracker *b, const Shape &sh, const std::vector<uint64_t *> &cols,
                const std::vector<int64_t> &n, Plan *out)
{
    Plan p;
    p.shape = sh;
    p.smem = track_smem_bytes(sh.stages, max_chunk_words(b));
    p.plain = true;
    for (const auto &v : b->views) p.plain = p.plain && plain_lattice(v.op_mask);
    int per_sm = 0;
    int rc = batch_ctas_per_sm(b->fast, p.plain, sh.threads, sh.blocks_per_sm, p.smem, &per_sm);
    if (rc != 0 || per_sm <= 0) {
        set_error("batch: launch shape does not fit an SM (threads " +
                  std::to_string(sh.threads) + ", stages " + std::to_string(sh.stages) + ")");
        return false;
    }
    p.grid = (unsigned)(b->sm_count * per_sm);
    size_t const V = b->views.size();
    std::vector<TrackParams> prm(V);
    std::vector<BatchItem> items;
    for (size_t v = 0; v < V; ++v) {
        const LatticeLaunchView &lv = b->views[v];
        TrackParams &t = prm[v];
        t = TrackParams{};
        t.stream = lv.stream;
        t.n_chunks = lv.n_chunks;
        t.chunk_words = lv.chunk_words;
        t.stages = sh.stages;
        t.mode = MODE_UNTIL;
        t.num_elements = lv.num_elements;
        t.cols = cols[v];
        t.n = n[v];
        t.i0 = 0;
        t.i1 = n[v];
        t.xlim_bits = lv.xlim_bits;
        t.ylim_bits = lv.ylim_bits;
        t.status = b->d_flags;
        t.error = b->d_flags + 1;
        t.s_table = lv.s_table;
        t.op_mask = lv.op_mask;
        if (lv.num_elements == 0) continue;  // nothing to apply
        for (int64_t f = 0; f < n[v]; f += sh.threads) items.push_back({(int32_t)v, 0, f});
    }
    // longest lattice first (ties: variant order, then particle order)
    std::stable_sort(items.begin(), items.end(), [&](const BatchItem &a, const BatchItem &c) {
        return b->views[a.variant].num_elements > b->views[c.variant].num_elements;
    });
    p.num_items = (int32_t)items.size();
    if (!cuda_ok(cudaMalloc(&p.d_variants, std::max<size_t>(V, 1) * sizeof(TrackParams)),
                 "cudaMalloc(batch variants)") ||
        !cuda_ok(cudaMalloc(&p.d_items, std::max<size_t>(items.size(), 1) * sizeof(BatchItem)),
                 "cudaMalloc(batch items)")) {
        p.release();
        return false;
    }
    if (!cuda_ok(cudaMemcpy(p.d_variants, prm.data(), V * sizeof(TrackParams),
                            cudaMemcpyHostToDevice),
                 "cudaMemcpy(batch variants)") ||
        (!items.empty() &&
         !cuda_ok(cudaMemcpy(p.d_items, items.data(), items.size() * sizeof(BatchItem),
                             cudaMemcpyHostToDevice),
                  "cudaMemcpy(batch items)"))) {
        p.release();
        return false;
    }
    *out = p;
    return true;
}

bool ensure_counters(st_BatchTracker *b, int64_t count)
{
    if (count <= b->n_counters) return true;
    if (b->d_counters) cudaFree(b->d_counters);
    b->d_counters = nullptr;
    b->n_counters = 0;
    if (!cuda_ok(cudaMalloc(&b->d_counters, (size_t)count * sizeof(int32_t)),
                 "cudaMalloc(batch counters)"))
        return false;
    b->n_counters = count;
    return true;
}

// Enqueue the launches that advance every variant by `turns` turns from
// *d_base, then advance *d_base.  Counters must hold ceil(turns / tpl).
bool enqueue_turns(st_BatchTracker *b, const Plan &p, int64_t turns, cudaStream_t s)
{
    int64_t const tpl = p.shape.turns_per_launch;
    int64_t const launches = (turns + tpl - 1) / tpl;
    if (!cuda_ok(cudaMemsetAsync(b->d_counters, 0, (size_t)launches * sizeof(int32_t), s),
                 "cudaMemsetAsync(batch counters)"))
        return false;
    for (int64_t k = 0; k < launches; ++k) {
        if (p.num_items == 0) break;
        BatchLaunch L{};
        L.variants = p.d_variants;
        L.items = p.d_items;
        L.num_items = p.num_items;
        L.counter = b->d_counters + k;
        L.base_turn = b->d_base;
        L.turn_offset = std::min(turns, (k + 1) * tpl);
        L.fast = b->fast;
        L.plain = p.plain;
        L.threads = p.shape.threads;
        L.blocks_per_sm = p.shape.blocks_per_sm;
        L.grid = p.grid;
        L.smem = p.smem;
        int const rc = launch_batch(L, s);
        if (rc != 0) {
            set_error(std::string("batch kernel launch: ") + cudaGetErrorString((cudaError_t)rc));
            return false;
        }
    }
    add_turn_kernel<<<1, 1, 0, s>>>(b->d_base, turns);
    if (!cuda_ok(cudaGetLastError(), "batch turn update")) return false;
    count_launches((uint64_t)(launches + 1));
    return true;
}

st_track_status_t read_status(st_BatchTracker *b, cudaStream_t s)
{
    if (!cuda_ok(cudaMemcpyAsync(b->h_flags, b->d_flags, 2 * sizeof(int32_t),
                                 cudaMemcpyDeviceToHost, s),
                 "cudaMemcpyAsync(batch status)") ||
        !cuda_ok(cudaStreamSynchronize(s), "batch kernel"))
        return -1;
    if (b->h_flags[1] != 0) {
        set_error("batch kernel: shared-memory pipeline wait timed out");
        return -1;
    }
    return b->h_flags[0];
}

void drop_graph(st_BatchTracker *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_turns = 0;
}

}  // namespace

extern "C" {

st_BatchTracker *st_BatchTracker_new(st_DeviceLattice *const *lattices, int32_t num_variants,
                                     const char *config)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    if (!lattices || num_variants <= 0) {
        set_error("batch: no lattices");
        return nullptr;
    }
    std::unique_ptr<st_BatchTracker> b(new st_BatchTracker());
    b->device = -1;
    std::string err;
    Shape sh;
    if (!parse_shape(config, &sh, &err) || !shape_valid(sh, &err)) {
        set_error(err);
        return nullptr;
    }
    b->views.resize((size_t)num_variants);
    for (int32_t v = 0; v < num_variants; ++v) {
        if (!device_lattice_view(lattices[v], &b->views[(size_t)v])) {
            set_error("batch: invalid lattice " + std::to_string(v));
            return nullptr;
        }
        const LatticeLaunchView &lv = b->views[(size_t)v];
        if (v == 0) {
            b->device = lv.device;
            b->fast = lv.fast;
        } else if (lv.device != b->device || lv.fast != b->fast) {
            set_error("batch: all lattices must be on one device with one arithmetic mode");
            return nullptr;
        }
    }
    if (!cuda_ok(cudaSetDevice(b->device), "cudaSetDevice") ||
        !cuda_ok(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device),
                 "cudaDeviceGetAttribute") ||
        !cuda_ok(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaMalloc(&b->d_base, sizeof(int64_t)), "cudaMalloc(batch turn)") ||
        !cuda_ok(cudaMalloc(&b->d_flags, 2 * sizeof(int32_t)), "cudaMalloc(batch status)") ||
        !cuda_ok(cudaMallocHost(&b->h_flags, 2 * sizeof(int32_t)), "cudaMallocHost"))
        return nullptr;
    b->plan.shape = sh;
    b->cols.assign((size_t)num_variants, nullptr);
    b->n.assign((size_t)num_variants, 0);
    return b.release();
}

void st_BatchTracker_delete(st_BatchTracker *b)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    delete b;
}

int32_t st_BatchTracker_set_particles(st_BatchTracker *b, void *const *d_cols,
                                      const int64_t *num_particles)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    if (!b || !d_cols || !num_particles) {
        set_error("batch: invalid arguments");
        return -1;
    }
    size_t const V = b->views.size();
    for (size_t v = 0; v < V; ++v) {
        if (num_particles[v] < 0 || (num_particles[v] > 0 && !d_cols[v])) {
            set_error("batch: bad particle block " + std::to_string(v));
            return -1;
        }
        if (num_particles[v] > 0 && b->views[v].num_elements == 0) {
            set_error("batch: variant " + std::to_string(v) + " has an empty lattice");
            return -1;
        }
        if (num_particles[v] > ((int64_t)1 << 40)) {
            set_error("batch: particle count out of range");
            return -1;
        }
    }
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    b->cols.assign(reinterpret_cast<uint64_t *const *>(d_cols),
                   reinterpret_cast<uint64_t *const *>(d_cols) + V);
    b->n.assign(num_particles, num_particles + V);
    Shape const sh = b->plan.shape;
    b->plan.release();
    drop_graph(b);
    return build_plan(b, sh, b->cols, b->n, &b->plan) ? 0 : -1;
}

st_track_status_t st_BatchTracker_track_until(st_BatchTracker *b, int64_t from_turn,
                                              int64_t until_turn, void *stream)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    if (!b || !b->plan.d_variants) {
        set_error("batch: particles not set");
        return -1;
    }
    cudaSetDevice(b->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (until_turn <= from_turn) return 0;
    int64_t const turns = until_turn - from_turn;
    int64_t const launches = (turns + b->plan.shape.turns_per_launch - 1) /
                             b->plan.shape.turns_per_launch;
    if (!ensure_counters(b, launches)) return -1;
    if (!cuda_ok(cudaMemsetAsync(b->d_flags, 0, 2 * sizeof(int32_t), s), "cudaMemsetAsync"))
        return -1;
    set_turn_kernel<<<1, 1, 0, s>>>(b->d_base, from_turn);
    if (!enqueue_turns(b, b->plan, turns, s)) return -1;
    return read_status(b, s);
}

int32_t st_BatchTracker_capture(st_BatchTracker *b, int64_t turns_per_replay)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    if (!b || !b->plan.d_variants || turns_per_replay <= 0) {
        set_error("batch: particles not set or bad turn count");
        return -1;
    }
    cudaSetDevice(b->device);
    int64_t const launches = (turns_per_replay + b->plan.shape.turns_per_launch - 1) /
                             b->plan.shape.turns_per_launch;
    if (!ensure_counters(b, launches)) return -1;
    drop_graph(b);
    if (!cuda_ok(cudaStreamSynchronize(b->stream), "batch stream") ||
        !cuda_ok(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal),
                 "cudaStreamBeginCapture"))
        return -1;
    bool ok = cuda_ok(cudaMemsetAsync(b->d_flags, 0, 2 * sizeof(int32_t), b->stream),
                      "cudaMemsetAsync") &&
              enqueue_turns(b, b->plan, turns_per_replay, b->stream);
    cudaGraph_t g = nullptr;
    cudaError_t const ec = cudaStreamEndCapture(b->stream, &g);
    if (!ok || !cuda_ok(ec, "cudaStreamEndCapture")) {
        if (g) cudaGraphDestroy(g);
        return -1;
    }
    b->graph = g;
    if (!cuda_ok(cudaGraphInstantiate(&b->exec, g, 0), "cudaGraphInstantiate")) {
        drop_graph(b);
        return -1;
    }
    b->graph_turns = turns_per_replay;
    return 0;
}

int32_t st_BatchTracker_set_turn(st_BatchTracker *b, int64_t turn, void *stream)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    if (!b) return -1;
    cudaSetDevice(b->device);
    set_turn_kernel<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(b->d_base, turn);
    return cuda_ok(cudaGetLastError(), "batch turn") ? 0 : -1;
}

int32_t st_BatchTracker_replay(st_BatchTracker *b, void *stream)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    if (!b || !b->exec) {
        set_error("batch: no captured graph");
        return -1;
    }
    cudaSetDevice(b->device);
    if (!cuda_ok(cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)), "cudaGraphLaunch"))
        return -1;
    count_launches((uint64_t)((b->graph_turns + b->plan.shape.turns_per_launch - 1) /
                                  b->plan.shape.turns_per_launch +
                              1));
    return 0;
}

st_track_status_t st_BatchTracker_status(st_BatchTracker *b, void *stream)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    if (!b) return -1;
    cudaSetDevice(b->device);
    return read_status(b, static_cast<cudaStream_t>(stream));
}

int32_t st_BatchTracker_get_shape(const st_BatchTracker *b, int32_t *threads,
                                  int32_t *blocks_per_sm, int32_t *stages,
                                  int32_t *turns_per_launch)
{
    if (!b) return -1;
    if (threads) *threads = b->plan.shape.threads;
    if (blocks_per_sm) *blocks_per_sm = b->plan.shape.blocks_per_sm;
    if (stages) *stages = b->plan.shape.stages;
    if (turns_per_launch) *turns_per_launch = b->plan.shape.turns_per_launch;
    return 0;
}

int32_t st_BatchTracker_autotune(st_BatchTracker *b, double sample_fraction, int64_t trial_turns,
                                 double *best_ms)
{
    DeviceGuard guard;  // the caller's current device is restored on return
    clear_error();
    if (!b || !b->plan.d_variants || trial_turns <= 0 || !(sample_fraction > 0.0)) {
        set_error("batch autotune: particles not set or bad arguments");
        return -1;
    }
    cudaSetDevice(b->device);
    cudaStream_t s = b->stream;
    size_t const V = b->views.size();
    // sample: the first ceil(n * fraction) particles of each variant (at
    // least one tile of the largest block size), copied out so the batch's
    // own particles are not touched
    std::vector<int64_t> ns(V);
    std::vector<size_t> off(V + 1, 0);
    for (size_t v = 0; v < V; ++v) {
        int64_t k = (int64_t)std::ceil((double)b->n[v] * std::min(sample_fraction, 1.0));
        k = std::min(b->n[v], std::max<int64_t>(k, kMaxThreads));
        ns[v] = k;
        off[v + 1] = off[v] + (size_t)k * 21;
    }
    uint64_t *pristine = nullptr, *work = nullptr;
    size_t const words = std::max<size_t>(off[V], 1);
    if (!cuda_ok(cudaMalloc(&pristine, words * 8), "cudaMalloc(autotune)") ||
        !cuda_ok(cudaMalloc(&work, words * 8), "cudaMalloc(autotune)")) {
        if (pristine) cudaFree(pristine);
        return -1;
    }
    bool ok = true;
    for (size_t v = 0; v < V && ok; ++v) {
        if (ns[v] == 0) continue;
        ok = cuda_ok(cudaMemcpy2DAsync(pristine + off[v], (size_t)ns[v] * 8, b->cols[v],
                                       (size_t)b->n[v] * 8, (size_t)ns[v] * 8, 21,
                                       cudaMemcpyDeviceToDevice, s),
                     "cudaMemcpy2DAsync(autotune sample)");
    }
    std::vector<uint64_t *> wcols(V);
    for (size_t v = 0; v < V; ++v) wcols[v] = work + off[v];
    // trials start from the earliest turn of a live sampled particle
    int64_t from = INT64_MAX;
    if (ok) {
        std::vector<int64_t> host(words);
        ok = cuda_ok(cudaMemcpyAsync(host.data(), pristine, words * 8, cudaMemcpyDeviceToHost, s),
                     "cudaMemcpyAsync(autotune sample)") &&
             cuda_ok(cudaStreamSynchronize(s), "autotune sample");
        for (size_t v = 0; v < V && ok; ++v)
            for (int64_t i = 0; i < ns[v]; ++i)
                if (host[off[v] + 20 * ns[v] + i] == 1)
                    from = std::min(from, host[off[v] + 19 * ns[v] + i]);
    }
    if (from == INT64_MAX) from = 0;
    int64_t const max_launches = trial_turns;
    ok = ok && ensure_counters(b, max_launches);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ok = ok && cuda_ok(cudaEventCreate(&e0), "cudaEventCreate") &&
         cuda_ok(cudaEventCreate(&e1), "cudaEventCreate");
    // time one shape on the sample (twice; the second run counts)
    auto trial = [&](const Shape &sh, double *ms) -> bool {
        Plan p;
        if (!build_plan(b, sh, wcols, ns, &p)) {
            clear_error();
            return false;  // shape does not fit: skipped
        }
        bool good = true;
        for (int rep = 0; rep < 2 && good; ++rep) {
            good = cuda_ok(cudaMemcpyAsync(work, pristine, words * 8, cudaMemcpyDeviceToDevice, s),
                           "cudaMemcpyAsync(autotune)");
            set_turn_kernel<<<1, 1, 0, s>>>(b->d_base, from);
            good = good && cuda_ok(cudaEventRecord(e0, s), "cudaEventRecord") &&
                   enqueue_turns(b, p, trial_turns, s) &&
                   cuda_ok(cudaEventRecord(e1, s), "cudaEventRecord") &&
                   cuda_ok(cudaEventSynchronize(e1), "autotune trial");
        }
        float t = 0.f;
        good = good && cuda_ok(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime");
        p.release();
        *ms = t;
        return good;
    };
    Shape best = b->plan.shape;
    double best_t = 1e300;
    if (ok) {
        double t;
        if (trial(best, &t)) best_t = t;
        // coordinate descent over the four knobs
        const int threads_c[] = {64, 128, 256};
        const int bpsm_c[] = {1, 2};
        const int stages_c[] = {2, 3, 4, 6, 8};
        const int tpl_c[] = {1, 2, 4, 8, 16};
        for (int pass = 0; pass < 2; ++pass) {
            for (int x : threads_c) {
                Shape c = best;
                c.threads = x;
                if (trial(c, &t) && t < best_t) best_t = t, best = c;
            }
            for (int x : bpsm_c) {
                Shape c = best;
                c.blocks_per_sm = x;
                if (trial(c, &t) && t < best_t) best_t = t, best = c;
            }
            for (int x : stages_c) {
                Shape c = best;
                c.stages = x;
                if (trial(c, &t) && t < best_t) best_t = t, best = c;
            }
            for (int x : tpl_c) {
                if (x > trial_turns) break;
                Shape c = best;
                c.turns_per_launch = x;
                if (trial(c, &t) && t < best_t) best_t = t, best = c;
            }
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(s);
    cudaFree(pristine);
    cudaFree(work);
    if (!ok || best_t >= 1e300) {
        if (ok) set_error("batch autotune: no launch shape could be timed");
        return -1;
    }
    Plan np;
    if (!build_plan(b, best, b->cols, b->n, &np)) return -1;
    b->plan.release();
    b->plan = np;
    drop_graph(b);
    if (best_ms) *best_ms = best_t;
    return 0;
}

}  // extern "C"

// track_kernel.cu -- the tracking kernel.
//
// One thread per particle; the particle's state lives in registers for the
// whole call (all turns).  The compiled element stream is staged into shared
// memory chunk by chunk with cp.async.bulk (the TMA engine's 1-D bulk copy)
// completing on mbarriers; every warp reads the records as broadcasts and
// dispatches on the opcode with a warp-uniform switch.  A lattice that fits
// the shared-memory stages is loaded once and stays resident for all turns;
// a longer one streams through the stages with STAGES-1 chunks in flight.
//
// Loop semantics follow the reference exactly:
//   until-turn      common/track/track.h:610-670
//   line            common/track/track.h:779-822
//   elem-by-elem    common/track/track.h:672-777
// (at_element_id is start + element ordinal while inside a turn and reset at
// the turn end, a failing or lost particle freezes where it stopped, status
// is OR-accumulated, -1 on failure).
//
// This translation unit is compiled with -fmad=false; the FAST instantiation
// uses explicit fma() (maps.cuh).
#include <cstdint>

#include "kernel_api.h"
#include "maps.cuh"

namespace stg {

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bulk (TMA) copy global -> shared, completion counted on `bar`.
// src and dst 16-byte aligned, bytes a multiple of 16 (chunks are).
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes,
                                              uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Bounded wait: gives up after ~2^31 clock cycles (~1 s) instead of hanging.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    long long const t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > (1ll << 31)) return false;
    }
    return true;
}

__device__ __forceinline__ void load_particle(PState &p, const uint64_t *cols, int64_t n,
                                              int64_t i)
{
    const double *d = reinterpret_cast<const double *>(cols);
    const int64_t *k = reinterpret_cast<const int64_t *>(cols);
    p.q0 = d[0 * n + i];
    p.mass0 = d[1 * n + i];
    p.beta0 = d[2 * n + i];
    p.gamma0 = d[3 * n + i];
    p.p0c = d[4 * n + i];
    p.s = d[5 * n + i];
    p.x = d[6 * n + i];
    p.y = d[7 * n + i];
    p.px = d[8 * n + i];
    p.py = d[9 * n + i];
    p.zeta = d[10 * n + i];
    p.psigma = d[11 * n + i];
    p.delta = d[12 * n + i];
    p.rpp = d[13 * n + i];
    p.rvv = d[14 * n + i];
    p.chi = d[15 * n + i];
    p.charge_ratio = d[16 * n + i];
    p.pid = k[17 * n + i];
    p.at_element = k[18 * n + i];
    p.at_turn = k[19 * n + i];
    p.state = k[20 * n + i];
    p.energy0 = sqrt(p.p0c * p.p0c + p.mass0 * p.mass0);
    refresh_kick_factors(p);
    p.lazy_s = false;
}

// Write one full record (21 columns) to a column block of capacity cap.
__device__ __forceinline__ void store_record(const PState &p, uint64_t *out, int64_t cap,
                                             int64_t j, int64_t at_element, int64_t at_turn,
                                             double s)
{
    double *d = reinterpret_cast<double *>(out);
    int64_t *k = reinterpret_cast<int64_t *>(out);
    d[0 * cap + j] = p.q0;
    d[1 * cap + j] = p.mass0;
    d[2 * cap + j] = p.beta0;
    d[3 * cap + j] = p.gamma0;
    d[4 * cap + j] = p.p0c;
    d[5 * cap + j] = s;
    d[6 * cap + j] = p.x;
    d[7 * cap + j] = p.y;
    d[8 * cap + j] = p.px;
    d[9 * cap + j] = p.py;
    d[10 * cap + j] = p.zeta;
    d[11 * cap + j] = p.psigma;
    d[12 * cap + j] = p.delta;
    d[13 * cap + j] = p.rpp;
    d[14 * cap + j] = p.rvv;
    d[15 * cap + j] = p.chi;
    d[16 * cap + j] = p.charge_ratio;
    k[17 * cap + j] = p.pid;
    k[18 * cap + j] = at_element;
    k[19 * cap + j] = at_turn;
    k[20 * cap + j] = p.state;
}

// be_monitor/track.h:48-110: output index for the current turn, or -1.
__device__ __forceinline__ int64_t monitor_index(const uint64_t *rec, int64_t turn, int64_t pid)
{
    int64_t const nstores = (int64_t)rec[1], start = (int64_t)rec[2], skip = (int64_t)rec[3];
    int64_t const max_pid = (int64_t)rec[4], min_pid = (int64_t)rec[5];
    int64_t const since = turn - start;
    int64_t out = -1;
    if (since >= 0 && (since % skip) == 0) {
        int64_t idx = since / skip;
        if (idx >= nstores && rec[6] != 0) idx = idx % nstores;
        if (idx < nstores) {
            int64_t const off = pid - min_pid;
            int64_t const np = max_pid - min_pid + 1;
            out = (rec[7] != 0) ? np * idx + off : off * np + idx;
        }
    }
    return out;
}

// output/elem_by_elem_config.h:667-763
__device__ __forceinline__ int64_t ebe_index(const EbeDevConfig &c, int64_t pid, int64_t elem,
                                             int64_t turn)
{
    int64_t out = -1;
    if (c.min_particle_id <= pid && c.max_particle_id >= pid && c.min_element_id <= elem &&
        c.max_element_id >= elem && c.min_turn <= turn &&
        (c.max_turn >= turn || c.is_rolling != 0)) {
        int64_t const np = c.num_particles_to_store, ne = c.num_elements_to_store;
        int64_t cap = 0;
        if (c.order == 0) {
            out = (turn - c.min_turn) * np * ne + (elem - c.min_element_id) * np +
                  (pid - c.min_particle_id);
            cap = np * ne * c.num_turns_to_store;
        }
        if (out >= cap && cap > 0 && c.is_rolling != 0) out = out % cap;
    }
    return out;
}

// Apply one element; returns 0 or -1 (reference status).  `lost` is set when
// the particle leaves the aperture (state becomes 0).  The PLAIN
// instantiation compiles only the maps of kPlainOps; the host chooses it
// for lattices without any other opcode, so its fall-through (failure,
// particle lost, as for an unknown type id) is never taken.
template <bool FAST, bool PLAIN, bool S_LIVE>
__device__ __forceinline__ int apply(PState &p, const uint64_t *rec, uint64_t hdr,
                                     const TrackParams &prm, int64_t cur_elem, int64_t cur_turn,
                                     int64_t ord)
{
    uint32_t const op = (uint32_t)(hdr & 0xFF);
    uint32_t const aux = (uint32_t)(hdr >> 32);
    switch (op) {
    case OP_DRIFT:
        drift<FAST, S_LIVE>(p, W(rec[1]));
        if (aux & DRIFT_APERTURE) p.state &= (int64_t)inside_global(p, prm.xlim_bits, prm.ylim_bits);
        return 0;
    case OP_MULTIPOLE:
        multipole<FAST, false>(p, rec, (int)aux);
        return 0;
    case OP_SROTATION:
        srotation<FAST>(p, rec);
        return 0;
    case OP_XYSHIFT:
        p.x += W(rec[1]);
        p.y += W(rec[2]);
        return 0;
    case OP_LIMIT_ELLIPSE:
        p.state &= (int64_t)inside_ellipse<FAST>(p, rec, aux);
        return 0;
    case OP_CAVITY:
        cavity(p, rec);
        return 0;
    case OP_MULTIPOLE_CURV:
        multipole<FAST, true>(p, rec, (int)aux);
        return 0;
    case OP_DRIFT_EXACT:
        drift_exact<S_LIVE>(p, W(rec[1]));
        if (aux & DRIFT_APERTURE) p.state &= (int64_t)inside_global(p, prm.xlim_bits, prm.ylim_bits);
        return 0;
    case OP_LIMIT_RECT:
        p.state &= (int64_t)inside_rect(p, rec);
        return 0;
    case OP_LIMIT_RECT_ELLIPSE:
        p.state &= (int64_t)inside_rect_ellipse(p, rec);
        return 0;
    case OP_DIPEDGE:
        p.px += W(rec[1]) * p.x;
        p.py += W(rec[2]) * p.y;
        return 0;
    case OP_RF_MULTIPOLE:
        if constexpr (PLAIN) break;
        else {
            p = rf_multipole(p, rec, (int)aux);
            return 0;
        }
    case OP_BB4D:
        if constexpr (PLAIN) break;
        else {
            p = beam_beam_4d(p, rec);
            return 0;
        }
    case OP_BB6D:
        if constexpr (PLAIN) break;
        else {
            if (aux & BB6D_ROUND)
                p = beam_beam_6d<true, FAST>(p, rec, (int)(aux & BB6D_SLICES));
            else
                p = beam_beam_6d<false, FAST>(p, rec, (int)aux);
            return 0;
        }
    case OP_SC_COASTING:
        if constexpr (PLAIN) break;
        else {
            p = sc_coasting(p, rec);
            return 0;
        }
    case OP_SC_QGAUSS:
        if constexpr (PLAIN) break;
        else {
            p = sc_qgauss<FAST>(p, rec, aux);
            return 0;
        }
    case OP_SC_INTERP:
        if constexpr (PLAIN) break;
        else {
            p = sc_interpolated(p, rec, aux);
            return 0;
        }
    case OP_TRICUB:
        if constexpr (PLAIN) break;
        else {
            p = tricub<FAST>(p, rec, aux);
            return p.state == 1 ? 0 : -1;  // outside the grid: lost, failure
        }
    case OP_MONITOR: {
        uint64_t *out = reinterpret_cast<uint64_t *>(rec[8]);
        if (out == nullptr) return 0;
        int64_t const j = monitor_index(rec, p.at_turn, p.pid);
        if (j < 0) return 0;
        if (j >= (int64_t)rec[9]) {
            p.state = 0;
            return -1;
        }
        store_record(p, out, (int64_t)rec[9], j, cur_elem, cur_turn,
                     p.lazy_s ? prm.s_table[ord] : p.s);
        return 0;
    }
    case OP_NOP:
        return 0;
    case OP_FAIL:
        return -1;
    default:  // OP_FAIL_LOST: unknown type id
        break;
    }
    p.state = 0;
    return -1;
}

}  // namespace

// The records of one staged chunk, in order, for the calling thread's
// particle (lanes whose particle takes no part are predicated off).
// S_LIVE (block-uniform for the pass): some particle of the block
// accumulates s, so drifts carry the s update.
template <bool FAST, bool PLAIN, bool S_LIVE>
__device__ __forceinline__ void walk_chunk(PState &p, const uint64_t *rec, const TrackParams &prm,
                                           bool &part, bool &active, int &status,
                                           int64_t &stop_elem, int64_t &ord, int64_t &ae,
                                           int64_t start_elem)
{
    while (true) {
        uint64_t const hdr = rec[0];
        uint32_t const nw = (uint32_t)((hdr >> 8) & 0xFFFFFF);
        if ((uint32_t)(hdr & 0xFF) == OP_END || nw == 0) break;
        if (part) {
            if (prm.mode == MODE_EBE) {
                int64_t const j = ebe_index(prm.ebe, p.pid, ae, p.at_turn);
                if (j >= 0 && j < prm.ebe_cap)
                    store_record(p, prm.ebe_out, prm.ebe_cap, j, ae, p.at_turn,
                                 p.lazy_s ? prm.s_table[ord] : p.s);
            }
            int const rc =
                apply<FAST, PLAIN, S_LIVE>(p, rec, hdr, prm, start_elem + ord, p.at_turn, ord);
            if (rc != 0 || p.state != 1) {
                status |= rc;
                part = false;
                active = false;
                stop_elem = ord;
                if (p.lazy_s) p.s = prm.s_table[ord + 1];
            } else {
                ++ae;
            }
        }
        ++ord;
        rec += nw;
    }
}

__device__ __forceinline__ void mbar_inval(uint64_t *bar)
{
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// One CTA's share of a tracking call: particle t of the launch (an index
// into prm.idx, or prm.i0 + t).  Block-uniform control flow: every thread
// walks every record of every chunk of every turn the block needs; lanes
// whose particle is done are predicated off inside apply().  `smem` holds
// 16 words of mbarriers followed by prm.stages chunk buffers.  Returns with
// every copy it issued complete; the caller invalidates the barriers before
// the shared memory is used again.
template <bool FAST, bool PLAIN>
__device__ __forceinline__ void track_block(const TrackParams &prm, int64_t t, uint64_t *smem)
{
    int const stages = prm.stages;
    int const cw = prm.chunk_words;
    uint64_t *bars = smem;                 // `stages` mbarriers (8 B each, padded to 16 words)
    uint64_t *bufs = smem + 16;            // stages * cw words
    __shared__ long long s_tmin;

    int64_t i;
    bool valid;
    if (prm.idx) {  // compacted launch: only the particles with work left
        valid = t < *prm.count;
        i = valid ? prm.idx[t] : 0;
    } else {
        i = prm.i0 + t;
        valid = i < prm.i1;
    }
    PState p;
    if (valid) {
        load_particle(p, prm.cols, prm.n, i);
        // s of a turn that starts at +0 comes from the lattice's s table
        p.lazy_s = (prm.mode != MODE_LINE) && (__double_as_longlong(p.s) == 0);
    }

    // ---------------------------------------------------- per-mode setup
    int64_t const start_elem = valid ? p.at_element : 0;
    bool active;   // still has work in this call
    if (prm.mode == MODE_UNTIL) {
        active = valid && p.state == 1 && p.at_turn < prm.until_turn;
    } else if (prm.mode == MODE_LINE) {
        active = valid && p.state == 1;
    } else {  // MODE_EBE: the reference does not check state here
        active = valid && prm.until_turn > p.at_turn && p.at_turn >= 0 && start_elem >= 0 &&
                 p.pid >= 0;
    }
    int status = 0;
    int64_t stop_elem = -1;  // element ordinal where tracking stopped
    bool const started = active;

    if (threadIdx.x == 0) {
        s_tmin = 0x7FFFFFFFFFFFFFFFll;
        for (int s = 0; s < stages; ++s) mbar_init(&bars[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (active && prm.mode != MODE_LINE) atomicMin(&s_tmin, (long long)p.at_turn);
    bool any = __syncthreads_or(active);
    int64_t turn = (prm.mode == MODE_LINE) ? 0 : (int64_t)s_tmin;

    int const nch = prm.n_chunks;
    bool const resident = nch <= stages;
    int64_t issued = 0;    // chunk loads issued (meaningful in thread 0 only)
    int64_t consumed = 0;  // chunk loads waited for (block-uniform)
    bool timed_out = false;
    if (any) {
        if (threadIdx.x == 0) {
            int const first = resident ? nch : stages;
            for (int g = 0; g < first; ++g) {
                mbar_arrive_expect_tx(&bars[g], (uint32_t)(cw * 8));
                bulk_copy_g2s(bufs + (size_t)g * cw, prm.stream + (size_t)(g % nch) * cw,
                              (uint32_t)(cw * 8), &bars[g]);
            }
            issued = first;
        }
        if (resident) {  // the whole lattice stays in shared memory
            // consumed = the first chunk not seen complete: after a timeout
            // the drain below waits for it and every later one
            int first_bad = nch;
            for (int g = 0; g < nch; ++g)
                if (!mbar_wait_bounded(&bars[g], 0u) && first_bad == nch) first_bad = g;
            consumed = first_bad;
            timed_out = __syncthreads_or(first_bad < nch);
        }
    }

    while (any && !timed_out) {
        bool part = (prm.mode == MODE_LINE) ? active : (active && (p.at_turn == turn));
        // some particle of the block accumulates s in this pass (block-uniform)
        bool const s_live = __syncthreads_or(part && !p.lazy_s);
        int64_t ord = 0;  // element ordinal within the turn / line
        int64_t ae = start_elem;
        for (int c = 0; c < nch; ++c) {
            int buf = c;
            if (!resident) {
                buf = (int)(consumed % stages);
                uint32_t const parity = (uint32_t)((consumed / stages) & 1);
                bool const ok = mbar_wait_bounded(&bars[buf], parity);
                if (ok) ++consumed;  // a chunk that timed out is left to the drain
                if (__syncthreads_or(!ok)) {
                    timed_out = true;
                    break;
                }
            }
            const uint64_t *rec = bufs + (size_t)buf * cw;
            if (s_live)
                walk_chunk<FAST, PLAIN, true>(p, rec, prm, part, active, status, stop_elem, ord,
                                              ae, start_elem);
            else
                walk_chunk<FAST, PLAIN, false>(p, rec, prm, part, active, status, stop_elem, ord,
                                               ae, start_elem);
            if (!resident) {
                __syncthreads();  // every warp is done with this stage buffer
                if (threadIdx.x == 0) {
                    int64_t const g = issued;  // next chunk of the cyclic stream
                    int const b = (int)(g % stages);
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_arrive_expect_tx(&bars[b], (uint32_t)(cw * 8));
                    bulk_copy_g2s(bufs + (size_t)b * cw, prm.stream + (size_t)(g % nch) * cw,
                                  (uint32_t)(cw * 8), &bars[b]);
                    issued = g + 1;
                }
            }
        }
        if (timed_out) break;
        if (prm.mode == MODE_LINE) {
            if (part && prm.finish_turn) {  // track/track.h:813-819
                p.at_turn += 1;
                p.s = 0.0;
            }
            active = false;
        } else if (part) {  // turn completed
            p.at_turn += 1;
            p.s = 0.0;
            p.lazy_s = true;
            if (p.at_turn >= prm.until_turn) active = false;
        }
        ++turn;
        any = __syncthreads_or(active);
        // every particle of the block is at a turn boundary here: a capped
        // launch may stop, the next launch resumes from the stored state
        if (prm.mode == MODE_UNTIL && prm.turn_cap > 0 && turn >= (int64_t)s_tmin + prm.turn_cap)
            any = false;
    }

    // drain bulk copies still in flight before the CTA exits (a resident
    // lattice has none left unless a wait timed out)
    if (threadIdx.x == 0 && (!resident || timed_out)) {
        while (consumed < issued) {
            int const buf = (int)(consumed % stages);
            uint32_t const parity = (uint32_t)((consumed / stages) & 1);
            if (!mbar_wait_bounded(&bars[buf], parity)) {
                timed_out = true;
                break;
            }
            ++consumed;
        }
    }
    if (timed_out) {
        if (threadIdx.x == 0) atomicOr(prm.error, ERR_PIPELINE_TIMEOUT);
        return;  // particle columns are left untouched
    }

    if (!valid) return;
    // ------------------------------------------------ final bookkeeping
    if (prm.mode == MODE_UNTIL) {
        if (stop_elem >= 0) {
            p.state = 0;  // track/track.h:663-666
            p.at_element = start_elem + stop_elem;
        }
    } else if (prm.mode == MODE_LINE) {
        if (started) {  // particles lost before the call are left as they are
            int64_t const done = (stop_elem >= 0) ? stop_elem : prm.num_elements;
            p.at_element = start_elem + done;
            if (stop_elem < 0 && prm.finish_turn && p.state == 1) p.at_element = 0;
        }
    } else {  // EBE
        if (stop_elem >= 0) p.at_element = start_elem + stop_elem;
    }
    if (status != 0) atomicOr(prm.status, status);

    double *d = reinterpret_cast<double *>(prm.cols);
    int64_t *k = reinterpret_cast<int64_t *>(prm.cols);
    int64_t const n = prm.n;
    d[5 * n + i] = p.s;
    d[6 * n + i] = p.x;
    d[7 * n + i] = p.y;
    d[8 * n + i] = p.px;
    d[9 * n + i] = p.py;
    d[10 * n + i] = p.zeta;
    d[11 * n + i] = p.psigma;
    d[12 * n + i] = p.delta;
    d[13 * n + i] = p.rpp;
    d[14 * n + i] = p.rvv;
    k[18 * n + i] = p.at_element;
    k[19 * n + i] = p.at_turn;
    k[20 * n + i] = p.state;
}

template <bool FAST, int MIN_BLOCKS, bool PLAIN>
__global__ void __launch_bounds__(kMaxThreads, MIN_BLOCKS) track_kernel(TrackParams prm)
{
    extern __shared__ __align__(128) uint64_t smem[];
    track_block<FAST, PLAIN>(prm, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, smem);
}

// Persistent batched kernel: each CTA takes work items (a tile of
// blockDim.x particles of one lattice variant) from a global counter until
// none is left, and tracks the tile until turn *base_turn + turn_offset with
// that variant's lattice.  Items are ordered longest first by the host.
template <bool FAST, int MIN_BLOCKS, bool PLAIN>
__global__ void __launch_bounds__(kMaxThreads, MIN_BLOCKS)
    batch_kernel(const TrackParams *variants, const BatchItem *items, int32_t num_items,
                 int32_t *counter, const int64_t *base_turn, int64_t turn_offset)
{
    extern __shared__ __align__(128) uint64_t smem[];
    __shared__ int32_t s_item;
    int64_t const until = *base_turn + turn_offset;
    while (true) {
        __syncthreads();  // previous item done (barriers invalidated, s_item read)
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        int32_t const it = s_item;
        if (it >= num_items) break;
        BatchItem const w = items[it];
        TrackParams prm = variants[w.variant];
        prm.until_turn = until;
        prm.idx = nullptr;
        prm.count = nullptr;
        prm.i0 = w.first;
        prm.i1 = (w.first + blockDim.x < prm.n) ? w.first + blockDim.x : prm.n;
        track_block<FAST, PLAIN>(prm, threadIdx.x, smem);
        __syncthreads();
        if (threadIdx.x == 0)
            for (int b = 0; b < prm.stages; ++b) mbar_inval(&smem[b]);
    }
}

#define STG_INSTANTIATE(F, M, P)                                                             \
    template __global__ void track_kernel<F, M, P>(TrackParams);                             \
    template __global__ void batch_kernel<F, M, P>(const TrackParams *, const BatchItem *,    \
                                                   int32_t, int32_t *, const int64_t *, int64_t);
STG_INSTANTIATE(false, 1, false)
STG_INSTANTIATE(true, 1, false)
STG_INSTANTIATE(false, 2, false)
STG_INSTANTIATE(true, 2, false)
STG_INSTANTIATE(false, 1, true)
STG_INSTANTIATE(true, 1, true)
STG_INSTANTIATE(false, 2, true)
STG_INSTANTIATE(true, 2, true)
#undef STG_INSTANTIATE

}  // namespace stg

namespace stg {

namespace {
__global__ void __launch_bounds__(256) exp_fast_kernel(const double *x, double *y, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = exp_fast(x[i]);
}
}  // namespace

namespace {
__global__ void __launch_bounds__(256) rcp_fast_kernel(const double *x, double *y, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        y[i] = rcp_fast(x[i]);
}
}  // namespace

int launch_rcp_fast(const double *x, double *y, int64_t n, void *stream)
{
    if (n <= 0) return 0;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    rcp_fast_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, y, n);
    return (int)cudaGetLastError();
}

int launch_exp_fast(const double *x, double *y, int64_t n, void *stream)
{
    if (n <= 0) return 0;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    exp_fast_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, y, n);
    return (int)cudaGetLastError();
}

size_t track_smem_bytes(int stages, int chunk_words)
{
    return (size_t)(16 + (size_t)stages * chunk_words) * sizeof(uint64_t);
}

template <bool FAST, int MB, bool PLAIN>
static int launch_one(const TrackParams &prm, unsigned blocks, int threads, size_t smem,
                      cudaStream_t s)
{
    cudaError_t err = cudaFuncSetAttribute(track_kernel<FAST, MB, PLAIN>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    track_kernel<FAST, MB, PLAIN><<<blocks, threads, smem, s>>>(prm);
    return (int)cudaGetLastError();
}

template <bool PLAIN>
static int launch_tier(const TrackParams &prm, bool fast, bool two, unsigned blocks, int threads,
                       size_t smem, cudaStream_t s)
{
    if (fast)
        return two ? launch_one<true, 2, PLAIN>(prm, blocks, threads, smem, s)
                   : launch_one<true, 1, PLAIN>(prm, blocks, threads, smem, s);
    return two ? launch_one<false, 2, PLAIN>(prm, blocks, threads, smem, s)
               : launch_one<false, 1, PLAIN>(prm, blocks, threads, smem, s);
}

int launch_track(const TrackParams &prm, bool fast, int threads, int blocks_per_sm, void *stream)
{
    int64_t const count = prm.i1 - prm.i0;
    if (count <= 0) return 0;
    if (threads <= 0 || threads > kMaxThreads || threads % 32 != 0) threads = kMaxThreads;
    int64_t const blocks = (count + threads - 1) / threads;
    size_t const smem = track_smem_bytes(prm.stages, prm.chunk_words);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    bool const two = blocks_per_sm >= 2;
    if (plain_lattice(prm.op_mask))
        return launch_tier<true>(prm, fast, two, (unsigned)blocks, threads, smem, s);
    return launch_tier<false>(prm, fast, two, (unsigned)blocks, threads, smem, s);
}

template <bool FAST, int MB, bool PLAIN>
static cudaError_t batch_occupancy(int threads, size_t smem, int *per_sm)
{
    cudaError_t err = cudaFuncSetAttribute(batch_kernel<FAST, MB, PLAIN>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, batch_kernel<FAST, MB, PLAIN>,
                                                         threads, smem);
}

template <bool PLAIN>
static cudaError_t batch_occupancy_tier(bool fast, bool two, int threads, size_t smem,
                                        int *per_sm)
{
    if (fast)
        return two ? batch_occupancy<true, 2, PLAIN>(threads, smem, per_sm)
                   : batch_occupancy<true, 1, PLAIN>(threads, smem, per_sm);
    return two ? batch_occupancy<false, 2, PLAIN>(threads, smem, per_sm)
               : batch_occupancy<false, 1, PLAIN>(threads, smem, per_sm);
}

int batch_ctas_per_sm(bool fast, bool plain, int threads, int blocks_per_sm, size_t smem,
                      int *per_sm)
{
    bool const two = blocks_per_sm >= 2;
    cudaError_t const err =
        plain ? batch_occupancy_tier<true>(fast, two, threads, smem, per_sm)
              : batch_occupancy_tier<false>(fast, two, threads, smem, per_sm);
    return (int)err;
}

int launch_batch(const BatchLaunch &b, void *stream)
{
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    bool const two = b.blocks_per_sm >= 2;
#define STG_BATCH(F, M, P)                                                                      \
    batch_kernel<F, M, P><<<b.grid, b.threads, b.smem, s>>>(b.variants, b.items, b.num_items,   \
                                                            b.counter, b.base_turn,              \
                                                            b.turn_offset)
    if (b.plain) {
        if (b.fast) {
            if (two) STG_BATCH(true, 2, true);
            else STG_BATCH(true, 1, true);
        } else {
            if (two) STG_BATCH(false, 2, true);
            else STG_BATCH(false, 1, true);
        }
    } else {
        if (b.fast) {
            if (two) STG_BATCH(true, 2, false);
            else STG_BATCH(true, 1, false);
        } else {
            if (two) STG_BATCH(false, 2, false);
            else STG_BATCH(false, 1, false);
        }
    }
#undef STG_BATCH
    return (int)cudaGetLastError();
}

}  // namespace stg

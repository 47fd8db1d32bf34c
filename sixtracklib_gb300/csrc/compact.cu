// compact.cu -- stable selection of the particles a tracking call must move.
//
// A warp of the tracking kernel issues every FP64 instruction for all 32
// lanes, live or not; with a beam that has lost part of its particles,
// lanes holding lost particles waste the (scarce) FP64 pipe.  Before a
// launch, the indices of the particles that still have work (state == 1 and,
// for until-turn tracking, at_turn < until_turn) are packed densely, in their
// original order, so the kernel's warps hold live particles only.
//
// Three passes over blocks of kSelBlock particles: count per block, exclusive
// scan of the block counts (one CTA), scatter of the indices.
#include <cstdint>

#include "kernel_api.h"

namespace stg {

namespace {

constexpr int kSelBlock = 1024;

__device__ __forceinline__ bool has_work(const uint64_t *cols, int64_t n, int64_t i, int mode,
                                         int64_t until)
{
    const int64_t *k = reinterpret_cast<const int64_t *>(cols);
    int64_t const state = k[20 * n + i];
    if (state != 1) return false;
    return mode == MODE_LINE || k[19 * n + i] < until;
}

__global__ void __launch_bounds__(kSelBlock) count_active(const uint64_t *cols, int64_t n,
                                                          int64_t i0, int64_t i1, int mode,
                                                          int64_t until, int32_t *counts)
{
    int64_t const i = i0 + (int64_t)blockIdx.x * kSelBlock + threadIdx.x;
    bool const a = (i < i1) && has_work(cols, n, i, mode, until);
    int const c = __syncthreads_count(a);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

// Exclusive scan of `nb` block counts by one CTA of kSelBlock threads.
__global__ void __launch_bounds__(kSelBlock) scan_counts(const int32_t *counts, int64_t nb,
                                                         int64_t *offsets, int64_t *total)
{
    __shared__ int64_t warp_sums[kSelBlock / 32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int64_t base = 0; base < nb; base += kSelBlock) {
        int64_t const j = base + threadIdx.x;
        int64_t v = (j < nb) ? counts[j] : 0;
        // inclusive warp scan
        int64_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t const y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int64_t w = warp_sums[lane];
            for (int o = 1; o < 32; o <<= 1) {
                int64_t const y = __shfl_up_sync(0xFFFFFFFFu, w, o);
                if (lane >= o) w += y;
            }
            warp_sums[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        int64_t const before_warp = (warp > 0) ? warp_sums[warp - 1] : 0;
        if (j < nb) offsets[j] = carry + before_warp + x - v;
        __syncthreads();
        if (threadIdx.x == kSelBlock - 1) carry += warp_sums[kSelBlock / 32 - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kSelBlock) scatter_active(const uint64_t *cols, int64_t n,
                                                            int64_t i0, int64_t i1, int mode,
                                                            int64_t until,
                                                            const int64_t *offsets, int64_t *idx)
{
    __shared__ int warp_base[kSelBlock / 32];
    int64_t const i = i0 + (int64_t)blockIdx.x * kSelBlock + threadIdx.x;
    bool const a = (i < i1) && has_work(cols, n, i, mode, until);
    unsigned const m = __ballot_sync(0xFFFFFFFFu, a);
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_base[warp] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < kSelBlock / 32; ++w) {
            int const c = warp_base[w];
            warp_base[w] = s;
            s += c;
        }
    }
    __syncthreads();
    if (a) {
        int const r = warp_base[warp] + __popc(m & ((1u << lane) - 1u));
        idx[offsets[blockIdx.x] + r] = i;
    }
}

}  // namespace

int64_t select_scratch_words(int64_t count)
{
    int64_t const nb = (count + kSelBlock - 1) / kSelBlock;
    // counts (int32, padded to words) + offsets + total + idx
    return (nb + 1) / 2 + nb + 1 + count + 4;
}

int launch_select(const uint64_t *cols, int64_t n, int64_t i0, int64_t i1, int mode,
                  int64_t until, uint64_t *scratch, int64_t **idx_out, int64_t **count_out,
                  void *stream)
{
    int64_t const count = i1 - i0;
    int64_t const nb = (count + kSelBlock - 1) / kSelBlock;
    int32_t *counts = reinterpret_cast<int32_t *>(scratch);
    int64_t *offsets = reinterpret_cast<int64_t *>(scratch + (nb + 1) / 2);
    int64_t *total = offsets + nb;
    int64_t *idx = total + 1;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nb == 0) {
        cudaMemsetAsync(total, 0, sizeof(int64_t), s);
    } else {
        count_active<<<(unsigned)nb, kSelBlock, 0, s>>>(cols, n, i0, i1, mode, until, counts);
        scan_counts<<<1, kSelBlock, 0, s>>>(counts, nb, offsets, total);
        scatter_active<<<(unsigned)nb, kSelBlock, 0, s>>>(cols, n, i0, i1, mode, until, offsets,
                                                          idx);
    }
    *idx_out = idx;
    *count_out = total;
    return (int)cudaGetLastError();
}

}  // namespace stg

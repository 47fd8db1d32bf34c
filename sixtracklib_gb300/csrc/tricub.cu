// tricub.cu -- per-cell coefficients of the TriCub field maps.
//
// NS(Track_particle_tricub) (be_tricub/track.h:51-224) gathers, for every
// particle and element, the 64 values around the particle's grid cell (f,
// df/dx, df/dy, df/dz, d2f/dxdy, d2f/dxdz, d2f/dydz, d3f/dxdydz at the eight
// corners, tricub_construct_b_vector at :226-262) and multiplies them by the
// inverse of the tricubic Hermite constraint matrix
// (NS(tricub_construct_coefs), be_tricub/coefficients.h) to get the 64
// polynomial coefficients.  The coefficients depend only on the cell, so
// they are computed here once per cell when the lattice is uploaded and the
// tracking kernel reads the cell's 64 values: an FP64 multiply-add chain of
// about a thousand operations per particle and element is paid once per
// cell instead.
//
// The constraint matrix is the Kronecker product of the 1-D cubic Hermite
// constraints (value and derivative at 0 and 1) in x, y and z, so its
// inverse is the Kronecker product of the 1-D inverse
//     c = H [f(0), f(1), f'(0), f'(1)],
//     H = {{1, 0, 0, 0}, {0, 0, 1, 0}, {-3, 3, -2, -1}, {2, -2, 1, 1}}
// (Lekien & Marsden, Int. J. Numer. Meth. Eng. 63 (2005) 455).  Entry
// (coefficient, corner value) is a product of three entries of H: an exact
// integer.  The reference's generated code adds, for every coefficient, the
// products entry * value of its nonzero entries in ascending order of the
// corner value, the first one assigned; each coefficient here is the same
// sum in the same order, every product and sum rounded separately (this
// translation unit is compiled with -fmad=false), so the coefficients are
// bit-identical to the reference's.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernel_api.h"

namespace stg {

namespace {

__device__ __forceinline__ int hermite(int row, int col)
{
    // H, columns f(0), f(1), f'(0), f'(1)
    switch (row) {
    case 0: return col == 0 ? 1 : 0;
    case 1: return col == 2 ? 1 : 0;
    case 2: return col == 0 ? -3 : col == 1 ? 3 : col == 2 ? -2 : -1;
    default: return col == 0 ? 2 : col == 1 ? -2 : 1;
    }
}

// Entry of the inverse constraint matrix for the coefficient of
// x^i y^j z^k (reference index r = i + 4 j + 16 k) and corner value
// v = 8 l + c: derivative kind l in the order f, x, y, z, xy, xz, yz, xyz;
// corner c with bit 0 / 1 / 2 = the upper node in x / y / z.
__device__ __forceinline__ int inverse_entry(int r, int v)
{
    int const l = v >> 3, c = v & 7;
    // derivative orders of kind l in x, y, z
    int const dxo = (l == 1 || l == 4 || l == 5 || l == 7) ? 1 : 0;
    int const dyo = (l == 2 || l == 4 || l == 6 || l == 7) ? 1 : 0;
    int const dzo = (l == 3 || l == 5 || l == 6 || l == 7) ? 1 : 0;
    return hermite(r & 3, 2 * dxo + (c & 1)) * hermite((r >> 2) & 3, 2 * dyo + ((c >> 1) & 1)) *
           hermite(r >> 4, 2 * dzo + (c >> 2));
}

// One thread per (cell, coefficient).  nodes: 8 values per node at
// l + 8 (ix + nx (iy + ny iz)) (tricub_construct_b_vector's indexing);
// cells: 64 coefficients per cell at cell = ix + (nx-1) (iy + (ny-1) iz),
// the coefficient of x^i y^j z^k at k + 4 j + 16 i (the tracking map reads
// them in that order).
__global__ void __launch_bounds__(256) tricub_cell_coefs(const double *__restrict__ nodes,
                                                         double *__restrict__ cells, int64_t nx,
                                                         int64_t ny, int64_t nz)
{
    int64_t const cx = nx - 1, cy = ny - 1;
    int64_t const total = cx * cy * (nz - 1) * 64;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        int64_t const cell = t >> 6;
        int const r = (int)(t & 63);
        int64_t const ix = cell % cx, iy = (cell / cx) % cy, iz = cell / (cx * cy);
        double acc = 0.0;
        bool first = true;
        for (int v = 0; v < 64; ++v) {
            int const a = inverse_entry(r, v);
            if (a == 0) continue;
            int const c = v & 7;
            int64_t const node = (ix + (c & 1)) + nx * ((iy + ((c >> 1) & 1)) + ny * (iz + (c >> 2)));
            double const term = (double)a * nodes[(v >> 3) + 8 * node];
            acc = first ? term : acc + term;
            first = false;
        }
        int const i = r & 3, j = (r >> 2) & 3, k = r >> 4;
        cells[cell * 64 + (k + 4 * j + 16 * i)] = acc;
    }
}

}  // namespace

int launch_tricub_cells(const double *nodes, double *cells, int64_t nx, int64_t ny, int64_t nz,
                        void *stream)
{
    if (nx < 2 || ny < 2 || nz < 2) return 0;
    int64_t const total = (nx - 1) * (ny - 1) * (nz - 1) * 64;
    int64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;  // grid-stride beyond 64 blocks per SM
    tricub_cell_coefs<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        nodes, cells, nx, ny, nz);
    return (int)cudaGetLastError();
}

}  // namespace stg

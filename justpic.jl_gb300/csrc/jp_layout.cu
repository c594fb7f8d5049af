// jp_layout.cu -- CellArray layout conversion between the GPU form
// (blocklength 0: component k of node c at c + nnodes * k) and the CPU form
// (blocklength 1: at k + ncomp * c), i.e. the permutedims(data, (3, 2, 1)) of
// src/CellArrays/conversion.jl:36-41 and ext/JustPICCUDAExt.jl:178-191.
//
// Both directions are the transpose of a row-major R x C matrix into C x R.
// Tiles of 32 x 32 elements go through shared memory so that the reads and the
// writes are both row-contiguous across a warp; a persistent grid walks the
// tiles. The kernel moves every byte once in and once out (HBM-bound).
#include "jp_internal.cuh"

namespace jp {

namespace {

constexpr int kTile = 32;
constexpr int kRows = 8;  // a block is 32 x 8 threads; each thread moves 4 elements of a tile

template <typename T>
__global__ void __launch_bounds__(kTile * kRows)
    transpose_kernel(const T* __restrict__ src, T* __restrict__ dst, int64_t R, int64_t C)
{
    __shared__ T tile[kTile][kTile + 1];
    const int64_t tiles_c = (C + kTile - 1) / kTile;
    const int64_t tiles = ((R + kTile - 1) / kTile) * tiles_c;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const int64_t r0 = (t / tiles_c) * kTile, c0 = (t % tiles_c) * kTile;
#pragma unroll
        for (int k = 0; k < kTile; k += kRows) {
            const int64_t r = r0 + ty + k, c = c0 + tx;
            if (r < R && c < C) tile[ty + k][tx] = src[r * C + c];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kTile; k += kRows) {
            const int64_t c = c0 + ty + k, r = r0 + tx;  // dst row c, column r
            if (c < C && r < R) dst[c * R + r] = tile[tx][ty + k];
        }
        __syncthreads();
    }
}

template <typename T>
cudaError_t transpose(const void* src, void* dst, int64_t R, int64_t C, cudaStream_t st)
{
    const int64_t tiles = ((R + kTile - 1) / kTile) * ((C + kTile - 1) / kTile);
    const int64_t cap = (int64_t)152 * 8;  // 152 SMs, 8 resident 256-thread blocks each
    const unsigned nb = (unsigned)(tiles < cap ? (tiles > 0 ? tiles : 1) : cap);
    transpose_kernel<T><<<nb, dim3(kTile, kRows), 0, st>>>((const T*)src, (T*)dst, R, C);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_cell_permute(jp_particles* P, const void* src, void* dst, int64_t nnodes, int ncomp,
                                int elem_bytes, bool to_cpu)
{
    // GPU form: ncomp rows of nnodes; CPU form: nnodes rows of ncomp
    const int64_t R = to_cpu ? ncomp : nnodes;
    const int64_t C = to_cpu ? nnodes : ncomp;
    if (R == 0 || C == 0) return cudaSuccess;
    switch (elem_bytes) {
        case 1: return transpose<uint8_t>(src, dst, R, C, P->stream);
        case 2: return transpose<uint16_t>(src, dst, R, C, P->stream);
        case 4: return transpose<uint32_t>(src, dst, R, C, P->stream);
        default: return transpose<uint64_t>(src, dst, R, C, P->stream);
    }
}

}  // namespace jp

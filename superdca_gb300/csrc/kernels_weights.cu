// kernels_weights.cu -- sequence reweighting on the GPU.
//
// SuperDCA's calculate_weights (SuperDCA/include/plmDCA_optimizer_parameters.hpp:
// 39-98) gives sequence i the weight mult_i / (mult_i + sum of mult_j over
// the other sequences j with identity (L - d_ij) / L >= threshold), d_ij
// the number of loci whose states differ.  That is N^2/2 Hamming distances
// over L loci (4.5 million pairs x 94,000 loci at 3000 x 94,000).
//
// Here the states are packed two bits per locus, 32 loci per 64-bit word;
// d_ij counts the 2-bit fields that differ ((a ^ b) | (a ^ b) >> 1, masked to
// the low bit of each field, popcount).  A CTA owns a 64 x 64 block of the
// lower triangle of the pair matrix, streams both sequence blocks through
// shared memory 32 words at a time and keeps 4 x 4 pair distances per thread
// in registers.  Distances are exact integers and the identity test is the
// reference's double comparison, so the weights are bit-identical.
#include <cstdint>

#include "engine.h"
#include "kernels_common.cuh"

namespace sdca {
namespace {

constexpr int WT = 64;      // sequences per tile side
constexpr int WCH = 32;     // words per shared-memory chunk
constexpr uint64_t LOWBITS = 0x5555555555555555ull;

// states [N][ld] u8 -> packed [N][W] u64
__global__ void k_pack2(const uint8_t *__restrict__ X, int64_t ld, int N, int L, int64_t W,
                        uint64_t *__restrict__ packed)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)N * W) return;
    const int64_t i = t / W, w = t % W;
    const uint8_t *row = X + i * ld + w * 32;
    uint64_t v = 0;
    for (int k = 0; k < 32; ++k) {
        const int64_t n = w * 32 + k;
        if (n < L) v |= (uint64_t)(row[k] & 3) << (2 * k);
    }
    packed[t] = v;
}

// DIST: write every pair's distance (both orders) instead of the neighbour sums
template <bool DIST>
__global__ void __launch_bounds__(256)
k_pair_neighbours(const uint64_t *__restrict__ packed, int N, int L, int64_t W, double threshold,
                  const double *__restrict__ mult, double *__restrict__ nbr,
                  unsigned long long *__restrict__ nonidentical, int32_t *__restrict__ dist)
{
    // lower-triangle tile index -> (ti, tj) with tj <= ti
    const int64_t tid = blockIdx.x;
    int ti = (int)((sqrt(8.0 * (double)tid + 1.0) - 1.0) / 2.0);
    while ((int64_t)ti * (ti + 1) / 2 > tid) --ti;
    while ((int64_t)(ti + 1) * (ti + 2) / 2 <= tid) ++ti;
    const int tj = (int)(tid - (int64_t)ti * (ti + 1) / 2);
    const int i0 = ti * WT, j0 = tj * WT;

    __shared__ uint64_t sa[WT][WCH + 1];
    __shared__ uint64_t sb[WT][WCH + 1];
    // 16 x 16 threads, 4 x 4 pairs each; rows interleaved by 16 so that the
    // shared-memory reads of a warp fall in distinct banks
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    int d[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) d[a][b] = 0;

    for (int64_t w0 = 0; w0 < W; w0 += WCH) {
        for (int k = threadIdx.x; k < WT * WCH; k += 256) {
            const int r = k / WCH, c = k % WCH;
            const int64_t w = w0 + c;
            const int ia = i0 + r, jb = j0 + r;
            sa[r][c] = (ia < N && w < W) ? packed[(int64_t)ia * W + w] : 0ull;
            sb[r][c] = (jb < N && w < W) ? packed[(int64_t)jb * W + w] : 0ull;
        }
        __syncthreads();
#pragma unroll 4
        for (int c = 0; c < WCH; ++c) {
            uint64_t av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = sa[ty + 16 * a][c];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = sb[tx + 16 * b][c];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const uint64_t x = av[a] ^ bv[b];
                    d[a][b] += __popcll((x | (x >> 1)) & LOWBITS);
                }
        }
        __syncthreads();
    }
    if (DIST) {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int i = i0 + ty + 16 * a;
            if (i >= N) continue;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int j = j0 + tx + 16 * b;
                if (j > i) continue;
                dist[(int64_t)i * N + j] = d[a][b];
                dist[(int64_t)j * N + i] = d[a][b];
            }
        }
        return;
    }
    unsigned long long nonid = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int i = i0 + ty + 16 * a;
        if (i >= N) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int j = j0 + tx + 16 * b;
            if (j >= i) continue;  // pairs j < i, as the reference loops
            const double identity = (double)(L - d[a][b]) / (double)L;
            if (identity >= threshold) {
                atomicAdd(nbr + i, mult ? mult[j] : 1.0);
                atomicAdd(nbr + j, mult ? mult[i] : 1.0);
            } else {
                ++nonid;
            }
        }
    }
    if (nonid) atomicAdd(nonidentical, nonid);
}

} // namespace

void launch_weights(const uint8_t *X, int64_t ld, int N, int L, uint64_t *packed, double threshold,
                    const double *mult, double *nbr, unsigned long long *nonidentical, cudaStream_t st)
{
    const int64_t W = (L + 31) / 32;
    const int64_t total = (int64_t)N * W;
    k_pack2<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(X, ld, N, L, W, packed);
    const int64_t nt = (N + WT - 1) / WT;
    const int64_t tiles = nt * (nt + 1) / 2;
    k_pair_neighbours<false><<<(unsigned)tiles, 256, 0, st>>>(packed, N, L, W, threshold, mult, nbr, nonidentical,
                                                              nullptr);
}

// the full N x N matrix of differing-locus counts (diagonal 0)
void launch_distances(const uint8_t *X, int64_t ld, int N, int L, uint64_t *packed, int32_t *dist, cudaStream_t st)
{
    const int64_t W = (L + 31) / 32;
    const int64_t total = (int64_t)N * W;
    k_pack2<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(X, ld, N, L, W, packed);
    const int64_t nt = (N + WT - 1) / WT;
    const int64_t tiles = nt * (nt + 1) / 2;
    k_pair_neighbours<true><<<(unsigned)tiles, 256, 0, st>>>(packed, N, L, W, 0.0, nullptr, nullptr, nullptr, dist);
}

} // namespace sdca

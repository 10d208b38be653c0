// kernels_tc.cu -- the tensor-core contraction form (tcgen05, sm_103a).
//
// Both contractions of an L-BFGS iteration are one-hot GEMMs, C = A . B^T with
// A the one-hot expansion of the alignment and B the per-slot operand:
//
//   forward   u[i][p*4+a]      = sum_{k=n*4+s} [X_in == s] * D_p[a][k]   (A: N x 4L)
//   backward  G[n*4+s][p*4+a]  = sum_i [X_in == s] * R_p[a][i]           (A: 4L x N)
//
// which are SuperDCA's gather (plmDCA_objective.hpp:86-121) and gradient
// scatter (plmDCA_objective.hpp:153-190) for a batch of target loci.
//
// Data path per CTA (128 x 128 output tile, K in steps of 64):
//   * warp 0, one thread: TMA loads of the u8 state tile (2 KB) and of the
//     fp16 hi and lo tiles of B (128 B swizzle), completing on full_raw[s];
//   * warps 2-5: expand the u8 tile to the fp16 one-hot A tile directly in the
//     128-byte-swizzled K-major layout the MMA reads (the one-hot matrix never
//     exists in HBM: 1 byte per locus is read instead of 8), fence to the async
//     proxy, arrive on full_a[s];
//   * warp 1, one thread: tcgen05.mma kind::f16 (M128 N128 K16, FP32
//     accumulators in TMEM): A x B_hi and then A x B_lo into the same
//     accumulator (or, with exact fp16 operands, a second N tile in the lo
//     slot); tcgen05.commit frees the stage;
//   * warps 2-5 again: tcgen05.ld the accumulator and store it, scaled back
//     by the per-slot power of two.
// With hi + lo operands the backward keeps the expanded A tiles in TMEM
// instead (tcgen05.st by the expansion warps, MMAs reading A from TMEM; see
// Cfg below).
// B is split as hi + lo fp16 halves of (value * 2^e) so that the product keeps
// about 22 significant bits; the one-hot A is exact in fp16.
//
// Every mbarrier wait is bounded: on timeout the kernel records an error code
// in *err and skips the remaining work instead of spinning.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "df.cuh"
#include "engine.h"
#include "kernels_common.cuh"
#include "tcgen05.cuh"

namespace sdca {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 64;
constexpr int A_BYTES = BM * BK * 2;   // one 128-row one-hot subtile
constexpr int B_BYTES = BN * BK * 2;   // one fp16 half (hi or lo) of the slot operand
constexpr int RAW_BYTES = 2048;        // u8 states behind one subtile
constexpr int THREADS = 192;

// A CTA owns MSUB consecutive 128-row subtiles and reuses each staged B tile
// for all of them: the slot operand is the traffic that the L2 has to carry,
// once per CTA per k-step.  TMEM holds one 128-column accumulator per subtile
// and N tile.  NT = 2 (slot operands exact in fp16, no lo half): the stage's
// lo slot carries a second N tile, so every expanded one-hot tile feeds two
// MMAs per K16 step, as it does for hi + lo.
//
// AT (backward only): the one-hot A tiles live in TMEM instead of shared
// memory.  The expansion warps write them with tcgen05.st (row m of a
// subtile in TMEM lane m, sequence pairs (2j, 2j+1) in column j as the low
// and high halves) and the MMAs read A from TMEM, so shared memory carries
// only the slot operand and the u8 state tiles: an M128 N128 K16 MMA with
// both operands in shared memory reads 8 KB per 64 cycles, which with the
// expansion's stores and the TMA writes is more than the 128 bytes per
// cycle shared memory delivers.  TMEM then holds the accumulators
// (MSUB x NT x 128 columns) and STG stages of MSUB A subtiles (32 columns
// each: 64 sequences).
template <int MSUB, int STG, int NT = 1, bool AT = false> struct Cfg {
    static constexpr int STAGE_BYTES = (AT ? 0 : MSUB * A_BYTES) + 2 * B_BYTES + MSUB * RAW_BYTES;
    static constexpr int SMEM_BYTES = STG * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
    static constexpr uint32_t ACC_COLS = MSUB * BN * NT;
    static constexpr uint32_t A_COLS = AT ? MSUB * (BK / 2) * STG : 0;
    static constexpr uint32_t TMEM_COLS = AT ? 512 : ACC_COLS;
    static_assert(STAGE_BYTES % 1024 == 0, "stage must keep 1024-byte alignment");
    static_assert(ACC_COLS + A_COLS <= 512, "TMEM holds 512 columns");
    static_assert(NT == 1 || NT == 2, "one or two N tiles per CTA");
};

enum { MODE_FWD = 0, MODE_BWD = 1 };

// instruction descriptor, kind::f16: A = B = F16, D = F32, K-major, M = 128, N = 128
constexpr uint32_t IDESC = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                        uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)
        : "memory");
}

// the same MMA with A read from TMEM (column tmem_a, lanes 0-127) and the
// instruction descriptor given (its N fitted to the tile's live columns)
__device__ __forceinline__ void mma_f16_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                           uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(tmem_d),
        "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// kind::f16 descriptor with N = the live columns of a tile rounded up to 16
// (at most BN): a partly filled last N tile issues only the MMA work it needs
__device__ __forceinline__ uint32_t idesc_fit(int cols)
{
    const int n = cols >= BN ? BN : (cols < 16 ? 16 : (cols + 15) / 16 * 16);
    return (IDESC & ~(0x3Fu << 17)) | ((uint32_t)(n >> 3) << 17);
}

// 32 consecutive TMEM columns of this warp's 32 lanes from 32 registers per thread
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
        "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]),
        "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]),
        "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
        : "memory");
}

// fp16 1.0 in lane s of four 16-bit lanes
__device__ __forceinline__ uint64_t onehot4(uint32_t s)
{
    return (uint64_t)0x3C00u << (16u * (s & 3u));
}

// forward: raw = 128 rows x 16 loci (u8); A row r = sequence, K = locus*4+state
__device__ __forceinline__ void expand_fwd(const uint8_t *raw, uint32_t a_base, int t)
{
    const uint4 w = *reinterpret_cast<const uint4 *>(raw + t * 16);
    const uint32_t words[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t wd = words[c >> 1];
        const uint32_t s0 = (wd >> (16 * (c & 1))) & 0xFF, s1 = (wd >> (16 * (c & 1) + 8)) & 0xFF;
        const uint64_t lo = onehot4(s0), hi = onehot4(s1);
        st_shared_v4(sw128(a_base, t, c),
                     make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi, (uint32_t)(hi >> 32)));
    }
}

// four bytes -> four fp16 lanes holding 1.0 where the byte equals s
__device__ __forceinline__ uint2 eq_halves(uint32_t bytes, uint32_t s4)
{
    const uint32_t m = __vcmpeq4(bytes, s4);  // 0xFF per equal byte
    const uint32_t a = __byte_perm(m, 0u, 0x1404) & 0x3C003C00u;
    const uint32_t b = __byte_perm(m, 0u, 0x3424) & 0x3C003C00u;
    return make_uint2(a, b);
}

// backward, A in TMEM: row t's 64 one-hot values as 32 sequence pairs
// (low half: the even sequence), the column order of the TMEM A operand
__device__ __forceinline__ void expand_bwd_regs(const uint8_t *raw, int t, uint32_t (&o)[32])
{
    const int nl = t >> 2;
    const uint32_t s4 = (uint32_t)(t & 3) * 0x01010101u;
    const uint4 *rp = reinterpret_cast<const uint4 *>(raw + nl * 64);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint4 w = rp[q];
        const uint2 e0 = eq_halves(w.x, s4), e1 = eq_halves(w.y, s4);
        const uint2 e2 = eq_halves(w.z, s4), e3 = eq_halves(w.w, s4);
        o[8 * q + 0] = e0.x;
        o[8 * q + 1] = e0.y;
        o[8 * q + 2] = e1.x;
        o[8 * q + 3] = e1.y;
        o[8 * q + 4] = e2.x;
        o[8 * q + 5] = e2.y;
        o[8 * q + 6] = e3.x;
        o[8 * q + 7] = e3.y;
    }
}

// backward: raw = 32 loci x 64 sequences (u8); A row r = locus*4+state, K = sequence
__device__ __forceinline__ void expand_bwd(const uint8_t *raw, uint32_t a_base, int t)
{
    const int nl = t >> 2;
    const uint32_t s4 = (uint32_t)(t & 3) * 0x01010101u;
    const uint4 *rp = reinterpret_cast<const uint4 *>(raw + nl * 64);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint4 w = rp[q];
        const uint2 e0 = eq_halves(w.x, s4), e1 = eq_halves(w.y, s4);
        const uint2 e2 = eq_halves(w.z, s4), e3 = eq_halves(w.w, s4);
        st_shared_v4(sw128(a_base, t, 2 * q), make_uint4(e0.x, e0.y, e1.x, e1.y));
        st_shared_v4(sw128(a_base, t, 2 * q + 1), make_uint4(e2.x, e2.y, e3.x, e3.y));
    }
}

struct GemmArgs {
    int mode;
    int kt_begin_stride;  // k-tiles per split
    int kt_total;
    int m_rows;           // valid output rows (N for forward, 4L for backward)
    int nlist;
    const int32_t *list;  // list position -> slot
    const SlotDev *sd;
    float inv_scale_fwd;  // unused when per-slot scales are read from sd
    // forward output: partial[split][slot][Nx] float4
    float4 *partial;
    int Bmax;
    int64_t Nx;
    // backward output: raw gradient into the slot's new-gradient buffer
    float *gpool;
    int64_t Dp;
    float inv_scale_bwd;
    int hi_only;          // the slot operand is exact in fp16 (its lo half is zero): skip the lo MMA
    // backward, max only: instead of writing the gradient, each slot's
    // max |g| over the blocks n != locus goes to gmax_acc[slot * gmax_stride]
    // (non-negative double bits, atomicMax)
    double *gmax_acc;
    int gmax_stride;
    // backward, digit planes: the list holds nslot slots and the B operand
    // planes x nslot virtual columns (plane d of list position s at virtual
    // position d * nslot + s); virtual position P is written to gpool buffer P
    int planes, nslot;
    int *err;
};

template <int MSUB, int STG, int NT, bool AT = false>
__global__ void __launch_bounds__(THREADS, 1)
k_gemm(const __grid_constant__ CUtensorMap tmRaw, const __grid_constant__ CUtensorMap tmBhi,
       const __grid_constant__ CUtensorMap tmBlo, const GemmArgs args)
{
    using C = Cfg<MSUB, STG, NT, AT>;
    constexpr int SB = C::STAGE_BYTES;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t sbase0 = smem_u32(smem_raw);
    const uint32_t sbase = (sbase0 + 1023u) & ~1023u;
    uint8_t *const sgen = smem_raw + (sbase - sbase0);
    const uint32_t bars = sbase + STG * SB;
    // stage layout: [A subtiles (not with AT) | B hi | B lo | raw u8 tiles]
    auto a_off = [](int ms) { return (uint32_t)(ms * A_BYTES); };
    constexpr uint32_t BHI = AT ? 0 : MSUB * A_BYTES, BLO = BHI + B_BYTES, RAW = BLO + B_BYTES;
    // barrier layout: full_raw[STG], full_a[STG], empty[STG], tmem_full, tmem addr
    auto full_raw = [&](int s) { return bars + 8u * s; };
    auto full_a = [&](int s) { return bars + 8u * (STG + s); };
    auto empty = [&](int s) { return bars + 8u * (2 * STG + s); };
    const uint32_t tmem_full = bars + 8u * (3 * STG);
    const uint32_t tmem_slot = bars + 8u * (3 * STG + 1);
    uint32_t *tmem_slot_gen = reinterpret_cast<uint32_t *>(sgen + STG * SB + 8 * (3 * STG + 1));

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m_group = blockIdx.x, n_tile = blockIdx.y * NT, split = blockIdx.z;   // first N tile
    const int kt0 = split * args.kt_begin_stride;
    const int kt1 = min(args.kt_total, kt0 + args.kt_begin_stride);
    const int nkt = max(0, kt1 - kt0);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STG; ++s) {
            mbar_init(full_raw(s), 1);
            mbar_init(full_a(s), 128);
            mbar_init(empty(s), 1);
        }
        mbar_init(tmem_full, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tmem_slot),
                     "r"(C::TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem_base = *tmem_slot_gen;
    bool failed = false;

    if (warp == 0) {
        if (lane == 0) {
            for (int j = 0; j < nkt; ++j) {
                const int s = j % STG;
                const uint32_t ph = (uint32_t)((j / STG) & 1);
                if (!mbar_wait(empty(s), ph ^ 1u)) { failed = true; break; }
                const uint32_t st = sbase + (uint32_t)s * SB;
                mbar_expect_tx(full_raw(s), MSUB * RAW_BYTES + (NT == 2 || !args.hi_only ? 2 : 1) * B_BYTES);
                const int kt = kt0 + j;
#pragma unroll
                for (int ms = 0; ms < MSUB; ++ms) {
                    const int mt = m_group * MSUB + ms;
                    if (args.mode == MODE_FWD)
                        tma_load_2d(st + RAW + ms * RAW_BYTES, &tmRaw, kt * 16, mt * BM, full_raw(s));
                    else
                        tma_load_2d(st + RAW + ms * RAW_BYTES, &tmRaw, kt * BK, mt * 32, full_raw(s));
                }
                tma_load_2d(st + BHI, &tmBhi, kt * BK, n_tile * BN, full_raw(s));
                if (NT == 2)   // the second N tile (rows past the operand's end read as zero)
                    tma_load_2d(st + BLO, &tmBhi, kt * BK, (n_tile + 1) * BN, full_raw(s));
                else if (!args.hi_only)
                    tma_load_2d(st + BLO, &tmBlo, kt * BK, n_tile * BN, full_raw(s));
            }
            // loads still in flight land before the block retires
            for (int j = max(0, nkt - STG); j < nkt; ++j)
                if (!mbar_wait(full_raw(j % STG), (uint32_t)((j / STG) & 1))) failed = true;
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // live columns of this CTA's N tiles (4 per list position)
            const int cols0 = 4 * args.nlist - n_tile * BN, cols1 = cols0 - BN;
            const uint32_t id0 = idesc_fit(cols0), id1 = idesc_fit(cols1);
            for (int j = 0; j < nkt; ++j) {
                const int s = j % STG;
                const uint32_t ph = (uint32_t)((j / STG) & 1);
                if (!mbar_wait(full_a(s), ph)) { failed = true; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t st = sbase + (uint32_t)s * SB;
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
                    const uint64_t bh = smem_desc_sw128(st + BHI + kk * 32);
                    const uint64_t bl = smem_desc_sw128(st + BLO + kk * 32);
#pragma unroll
                    for (int ms = 0; ms < MSUB; ++ms) {
                        const uint32_t td = tmem_base + (uint32_t)(ms * BN);
                        if (AT) {
                            // K16 step kk: 8 of the subtile's 32 A columns
                            const uint32_t ta =
                                tmem_base + C::ACC_COLS + (uint32_t)((s * MSUB + ms) * (BK / 2) + kk * 8);
                            mma_f16_ts(td, ta, bh, id0, (j > 0 || kk > 0) ? 1u : 0u);
                            if (NT == 2) {
                                if (cols1 > 0)   // (a second tile with no live column is not computed)
                                    mma_f16_ts(td + (uint32_t)(MSUB * BN), ta, bl, id1, (j > 0 || kk > 0) ? 1u : 0u);
                            } else if (!args.hi_only) {
                                mma_f16_ts(td, ta, bl, id0, 1u);
                            }
                        } else {
                            const uint64_t ad = smem_desc_sw128(st + a_off(ms) + kk * 32);
                            mma_f16(td, ad, bh, (j > 0 || kk > 0) ? 1u : 0u);
                            if (NT == 2)
                                mma_f16(td + (uint32_t)(MSUB * BN), ad, bl, (j > 0 || kk > 0) ? 1u : 0u);
                            else if (!args.hi_only)
                                mma_f16(td, ad, bl, 1u);
                        }
                    }
                }
                mma_commit(empty(s));
            }
            // the accumulators are complete (or abandoned) once every issued MMA retired
            mma_commit(tmem_full);
        }
    } else {
        // with AT a warp writes only its TMEM lane quadrant: row = 32 (warp % 4) + lane
        const int t = AT ? 32 * (warp & 3) + lane : threadIdx.x - 64;  // 0..127
        for (int j = 0; j < nkt; ++j) {
            const int s = j % STG;
            const uint32_t ph = (uint32_t)((j / STG) & 1);
            // (full_raw(s) completes only after the producer saw empty(s): the
            // MMAs that read this stage's A before have retired)
            if (!mbar_wait(full_raw(s), ph)) { failed = true; break; }
            const uint32_t st = sbase + (uint32_t)s * SB;
#pragma unroll
            for (int ms = 0; ms < MSUB; ++ms) {
                const uint8_t *raw = sgen + s * SB + RAW + ms * RAW_BYTES;
                if (AT) {
                    uint32_t o[32];
                    expand_bwd_regs(raw, t, o);
                    tmem_st32(tmem_base + ((uint32_t)(32 * (warp & 3)) << 16) + C::ACC_COLS +
                                  (uint32_t)((s * MSUB + ms) * (BK / 2)),
                              o);
                } else if (args.mode == MODE_FWD) {
                    expand_fwd(raw, st + a_off(ms), t);
                } else {
                    expand_bwd(raw, st + a_off(ms), t);
                }
            }
            if (AT) {
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            } else {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            }
            mbar_arrive(full_a(s));
        }
        // epilogue
        const bool ok = nkt > 0 && mbar_wait(tmem_full, 0u);
        if (!ok && nkt > 0) failed = true;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int q = warp & 3;  // TMEM lane quadrant of this warp
        const int r = q * 32 + lane;
#pragma unroll 1
        for (int nm = 0; nm < NT * MSUB; ++nm) {
            const int nt = nm / MSUB, ms = nm % MSUB;
            const uint32_t tbase = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(nm * BN);
            const int row = (m_group * MSUB + ms) * BM + r;
#pragma unroll 1
            for (int cj = 0; cj < BN / 32; ++cj) {
                float v[32];
                if (ok) tmem_ld32(tbase + (uint32_t)(cj * 32), v);
                if (!ok) continue;
#pragma unroll
                for (int tt = 0; tt < 8; ++tt) {
                    const int P = ((n_tile + nt) * BN + cj * 32) / 4 + tt;
                    if (P >= args.nlist) continue;
                    const int b = args.planes > 1 ? args.list[P % args.nslot] : args.list[P];
                    if (args.mode == MODE_FWD) {
                        if (row < args.Nx) {
                            const float sc = (float)args.sd[b].tc_inv_scale;
                            args.partial[((int64_t)split * args.Bmax + b) * args.Nx + row] =
                                make_float4(v[4 * tt] * sc, v[4 * tt + 1] * sc, v[4 * tt + 2] * sc,
                                            v[4 * tt + 3] * sc);
                        }
                    } else if (args.gmax_acc) {
                        // (the list position P is the same in every lane of the warp)
                        float mv = 0.f;
                        if (row < args.m_rows && (row >> 2) != args.sd[b].locus)
                            mv = fmaxf(fmaxf(fabsf(v[4 * tt]), fabsf(v[4 * tt + 1])),
                                       fmaxf(fabsf(v[4 * tt + 2]), fabsf(v[4 * tt + 3]))) * args.inv_scale_bwd;
                        const unsigned mask = __activemask();
                        const unsigned mb = __reduce_max_sync(mask, __float_as_uint(mv));
                        if (lane == __ffs(mask) - 1 && mb != 0u)
                            atomicMax(reinterpret_cast<unsigned long long *>(args.gmax_acc +
                                                                             (int64_t)b * args.gmax_stride),
                                      (unsigned long long)__double_as_longlong((double)__uint_as_float(mb)));
                    } else if (row < args.m_rows) {
                        const float sc = args.inv_scale_bwd;
                        const int64_t buf = args.planes > 1 ? (int64_t)P : (int64_t)(2 * b + 1 - args.sd[b].gcur);
                        float *gn = args.gpool + buf * args.Dp + (int64_t)(row >> 2) * QQ + (row & 3) * Q;
                        *reinterpret_cast<float4 *>(gn) = make_float4(v[4 * tt] * sc, v[4 * tt + 1] * sc,
                                                                      v[4 * tt + 2] * sc, v[4 * tt + 3] * sc);
                    }
                }
            }
        }
    }
    if (failed) atomicExch(args.err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(C::TMEM_COLS)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// Exact K rho for the dual form on the tensor cores.
//
// K (agreement counts, < 2^18) is held as three fp16 planes of base-64
// digits (0..63), rho_q (integers, |rho_q| <= 2^27) as four fp16 planes of
// balanced base-128 digits (|digit| <= 64, the top one <= 65).  Every product
// of two digits is an integer below 4096 and the sum over at most 4000
// sequences stays below 2^24, so each of the 12 digit-pair GEMMs is exact in
// its FP32 TMEM accumulator; the epilogue combines them with their weights
// 2^(6k + 7p) in 64-bit integers (modulo 2^64: the total is below 2^62).
//
// Every row of rho_q sums to zero (k_dual_quant makes it so exactly), so the
// fourth column of K rho is minus the sum of the other three: only three
// columns per slot enter the product.  A CTA takes 128 rows of K and 13
// slots (39 columns; with one unused row, 40 rows per rho digit plane), the
// most that the 12 accumulators leave room for in TMEM (3 K digits x 4 planes
// x 40 columns = 480 of 512), so each K tile staged from L2 serves 13 slots.
// The B operand of one MMA stacks the four planes' first 32 rows (4 x 4 KB)
// and then their last 8 rows (4 x 1 KB): every plane's accumulator columns
// start 32-aligned (x32 loads) and its tail 8-aligned (x8 loads).

constexpr int KD_BM = 128, KD_BK = 64;
constexpr int KD_KDIG = 3, KD_RDIG = 4;
constexpr int KD_S = 13;                     // slots per CTA
constexpr int KD_C = 3;                      // product columns per slot (the fourth follows)
constexpr int KD_COLS = KD_S * KD_C;         // 39 live columns per plane
constexpr int KD_BN = 40;                    // rows per rho digit plane in a B tile
constexpr int KD_HEAD = 32, KD_TAIL = KD_BN - KD_HEAD;
constexpr int KD_A_BYTES = KD_BM * KD_BK * 2;          // one K digit plane tile, 16 KB
constexpr int KD_HEAD_BYTES = KD_HEAD * KD_BK * 2;     // 4 KB
constexpr int KD_TAIL_BYTES = KD_TAIL * KD_BK * 2;     // 1 KB
constexpr int KD_STAGE = KD_KDIG * KD_A_BYTES + KD_RDIG * (KD_HEAD_BYTES + KD_TAIL_BYTES);
constexpr int KD_STG = 3;
constexpr int KD_SMEM = KD_STG * KD_STAGE + 1024 + 256;
constexpr uint32_t KD_TMEM_COLS = 512;
constexpr int KD_NB = KD_RDIG * KD_BN;                 // 160 accumulator columns per K digit
constexpr uint32_t IDESC_KD = (1u << 4) | ((uint32_t)(KD_NB >> 3) << 17) | ((uint32_t)(KD_BM >> 4) << 24);
static_assert(KD_STAGE % 1024 == 0, "stage must keep 1024-byte alignment");
static_assert(KD_HEAD_BYTES % 1024 == 0 && KD_TAIL_BYTES % 1024 == 0, "TMA destinations 1024-aligned");
static_assert(KD_TAIL == 0 || KD_TAIL == 8, "plane tails of 8 rows (or none)");
static_assert(KD_KDIG * KD_NB <= (int)KD_TMEM_COLS, "accumulators fit TMEM");
static_assert(KD_NB % 16 == 0 && KD_NB <= 256, "MMA N for M = 128");
static_assert(KD_COLS < KD_BN, "one unused row per plane");

__device__ __forceinline__ void mma_f16_kd(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(IDESC_KD), "r"(accumulate)
        : "memory");
}

struct KdArgs {
    int kt_total;        // Nx / 64
    int nk_rows;         // rows per K digit plane (multiple of 128)
    int nr_rows;         // rows per rho digit plane (>= 3 x slots + 1)
    int N;
    int64_t Nx;
    int nlist;
    const int32_t *list;
    const uint8_t *rstate;
    const long long *csum;
    double inv_qscale;
    float2 *KR;                  // K rho / qscale in double-float
    int *err;
    const int *ncount;           // list length in device memory (the grid covers the most slots), or null
};

__global__ void __launch_bounds__(THREADS, 1)
k_kdig(const __grid_constant__ CUtensorMap tmK, const __grid_constant__ CUtensorMap tmRh,
       const __grid_constant__ CUtensorMap tmRt, const KdArgs args)
{
    extern __shared__ uint8_t smem_raw[];
    const uint32_t sbase0 = smem_u32(smem_raw);
    const uint32_t sbase = (sbase0 + 1023u) & ~1023u;
    uint8_t *const sgen = smem_raw + (sbase - sbase0);
    const uint32_t bars = sbase + KD_STG * KD_STAGE;
    auto full = [&](int s) { return bars + 8u * s; };
    auto empty = [&](int s) { return bars + 8u * (KD_STG + s); };
    const uint32_t tmem_full = bars + 8u * (2 * KD_STG);
    const uint32_t tmem_slot = bars + 8u * (2 * KD_STG + 1);
    uint32_t *tmem_slot_gen = reinterpret_cast<uint32_t *>(sgen + KD_STG * KD_STAGE + 8 * (2 * KD_STG + 1));
    constexpr uint32_t BOFF = KD_KDIG * KD_A_BYTES;                      // plane heads
    constexpr uint32_t TOFF = BOFF + KD_RDIG * KD_HEAD_BYTES;            // plane tails

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m_tile = blockIdx.x, n_tile = blockIdx.y;
    const int nkt = args.kt_total;
    const int nlist = args.ncount ? *args.ncount : args.nlist;
    if (n_tile * KD_S >= nlist) return;   // (the whole CTA, before any barrier or TMEM allocation)

    if (threadIdx.x == 0) {
        for (int s = 0; s < KD_STG; ++s) {
            mbar_init(full(s), 1);
            mbar_init(empty(s), 1);
        }
        mbar_init(tmem_full, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tmem_slot),
                     "r"(KD_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem_base = *tmem_slot_gen;
    bool failed = false;

    if (warp == 0) {
        if (lane == 0) {
            const int r0 = n_tile * KD_COLS;   // this CTA's first rho row in each plane
            for (int j = 0; j < nkt; ++j) {
                const int s = j % KD_STG;
                const uint32_t ph = (uint32_t)((j / KD_STG) & 1);
                if (!mbar_wait(empty(s), ph ^ 1u)) { failed = true; break; }
                const uint32_t st = sbase + (uint32_t)s * KD_STAGE;
                mbar_expect_tx(full(s), KD_STAGE);
#pragma unroll
                for (int k = 0; k < KD_KDIG; ++k)
                    tma_load_2d(st + k * KD_A_BYTES, &tmK, j * KD_BK, k * args.nk_rows + m_tile * KD_BM, full(s));
#pragma unroll
                for (int p = 0; p < KD_RDIG; ++p) {
                    tma_load_2d(st + BOFF + p * KD_HEAD_BYTES, &tmRh, j * KD_BK, p * args.nr_rows + r0, full(s));
                    if (KD_TAIL > 0)
                        tma_load_2d(st + TOFF + p * KD_TAIL_BYTES, &tmRt, j * KD_BK, p * args.nr_rows + r0 + KD_HEAD,
                                    full(s));
                }
            }
            for (int j = max(0, nkt - KD_STG); j < nkt; ++j)
                if (!mbar_wait(full(j % KD_STG), (uint32_t)((j / KD_STG) & 1))) failed = true;
        }
    } else if (warp == 1) {
        if (lane == 0) {
            for (int j = 0; j < nkt; ++j) {
                const int s = j % KD_STG;
                const uint32_t ph = (uint32_t)((j / KD_STG) & 1);
                if (!mbar_wait(full(s), ph)) { failed = true; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t st = sbase + (uint32_t)s * KD_STAGE;
#pragma unroll
                for (int kk = 0; kk < KD_BK / 16; ++kk) {
                    const uint64_t bd = smem_desc_sw128(st + BOFF + kk * 32);
#pragma unroll
                    for (int k = 0; k < KD_KDIG; ++k) {
                        const uint64_t ad = smem_desc_sw128(st + k * KD_A_BYTES + kk * 32);
                        mma_f16_kd(tmem_base + (uint32_t)(k * KD_NB), ad, bd, (j > 0 || kk > 0) ? 1u : 0u);
                    }
                }
                mma_commit(empty(s));
            }
            mma_commit(tmem_full);
        }
    } else {
        const bool ok = nkt > 0 && mbar_wait(tmem_full, 0u);
        if (!ok && nkt > 0) failed = true;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int q = warp & 3;
        const int row = m_tile * KD_BM + q * 32 + lane;
        const float2 iq = df_from_d(args.inv_qscale);
        // The 12 digit products are integers below 2^24 in magnitude (exact
        // in the FP32 accumulators): each is converted with a 32-bit
        // conversion and shifted into place in 64-bit integers (no 64-bit
        // conversion or multiply, which run on GB300's narrow FP64 pipe).
        long long acc[KD_COLS];
#pragma unroll
        for (int c = 0; c < KD_COLS; ++c) acc[c] = 0ll;
        if (ok) {
            const uint32_t lanes = (uint32_t)(q * 32) << 16;
#pragma unroll 1
            for (int k = 0; k < KD_KDIG; ++k)
#pragma unroll 1
                for (int p = 0; p < KD_RDIG; ++p) {
                    const int sh = 6 * k + 7 * p;
                    float v[32], t[8] = {};
                    tmem_ld32(tmem_base + lanes + (uint32_t)(k * KD_NB + p * KD_HEAD), v);
                    if (KD_TAIL > 0)
                        tmem_ld8(tmem_base + lanes + (uint32_t)(k * KD_NB + KD_RDIG * KD_HEAD + p * KD_TAIL), t);
#pragma unroll
                    for (int c = 0; c < (KD_HEAD < KD_COLS ? KD_HEAD : KD_COLS); ++c)
                        acc[c] += (long long)__float2int_rn(v[c]) << sh;
#pragma unroll
                    for (int c = KD_HEAD; c < KD_COLS; ++c) acc[c] += (long long)__float2int_rn(t[c - KD_HEAD]) << sh;
                }
#pragma unroll
            for (int s = 0; s < KD_S; ++s) {
                const int P = n_tile * KD_S + s;
                if (P >= nlist || row >= args.Nx) continue;
                const int b = args.list[P];
                float2 val[4] = {df_zero(), df_zero(), df_zero(), df_zero()};
                if (row < args.N) {
                    const int y = args.rstate[(int64_t)b * args.Nx + row] & 3;
                    const long long *cs = args.csum + (int64_t)b * 16 + y * 4;
                    long long tot[4];
#pragma unroll
                    for (int c = 0; c < KD_C; ++c) tot[c] = acc[KD_C * s + c] - cs[c];
                    tot[3] = -(tot[0] + tot[1] + tot[2]);
#pragma unroll
                    for (int c = 0; c < 4; ++c) val[c] = df_mul(df_from_ll_fast(tot[c]), iq);
                }
                float4 *o = reinterpret_cast<float4 *>(args.KR + ((int64_t)b * args.Nx + row) * 4);
                o[0] = make_float4(val[0].x, val[0].y, val[1].x, val[1].y);
                o[1] = make_float4(val[2].x, val[2].y, val[3].x, val[3].y);
            }
        }
    }
    if (failed) atomicExch(args.err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(KD_TMEM_COLS)
                     : "memory");
    }
}

// K (int32, Nx x Nx) -> three fp16 planes of base-64 digits, rows padded to nk_rows
__global__ void k_kdig_split_k(const int32_t *__restrict__ K, int64_t Nx, int nk_rows, __half *__restrict__ Kd)
{
    const int64_t total = (int64_t)nk_rows * Nx;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / Nx;
        const int v = i < Nx ? K[t] : 0;
        Kd[t] = __int2half_rn(v & 63);
        Kd[(int64_t)nk_rows * Nx + t] = __int2half_rn((v >> 6) & 63);
        Kd[2 * (int64_t)nk_rows * Nx + t] = __int2half_rn(v >> 12);
    }
}

// rho_q of list position P (slot list[P]), its first three columns -> four
// fp16 planes of balanced base-128 digits, rows P*3+c
__global__ void k_kdig_split_r(const int32_t *__restrict__ list, int64_t Nx, int nr_rows,
                               const int4 *__restrict__ rq, __half *__restrict__ Rd, const int *__restrict__ cnt)
{
    if (cnt && (int)blockIdx.y >= *cnt) return;
    const int P = blockIdx.y, b = list[P];
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < Nx; j += (int64_t)gridDim.x * blockDim.x) {
        const int4 q = rq[(int64_t)b * Nx + j];
        const int qq[KD_C] = {q.x, q.y, q.z};
#pragma unroll
        for (int c = 0; c < KD_C; ++c) {
            long long v = qq[c];
#pragma unroll
            for (int p = 0; p < KD_RDIG; ++p) {
                long long d = v;
                if (p < KD_RDIG - 1) {
                    d = ((v + 64) & 127) - 64;   // balanced digit, v - d divisible by 128
                    v = (v - d) / 128;
                }
                Rd[((int64_t)p * nr_rows + (int64_t)P * KD_C + c) * Nx + j] = __int2half_rn((int)d);
            }
        }
    }
}

// d (engine layout [n][s][a]) -> B rows p*4+a, columns n*4+s, fp16 hi and lo of d*2^e
__global__ void k_split_dir(const SlotDev *__restrict__ sd, const int32_t *__restrict__ list, int64_t L,
                            int64_t Dp, int64_t Kp, const float *__restrict__ vecs, __half *__restrict__ hi,
                            __half *__restrict__ lo)
{
    const int P = blockIdx.y;
    const int b = list[P];
    const float sc = (float)sd[b].tc_scale;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < 4 * L; k += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = *reinterpret_cast<const float4 *>(vecs + (int64_t)b * Dp + k * 4);
        const float vv[4] = {v.x * sc, v.y * sc, v.z * sc, v.w * sc};
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const __half h = __float2half_rn(vv[a]);
            const __half l = __float2half_rn(vv[a] - __half2float(h));
            const int64_t o = ((int64_t)P * 4 + a) * Kp + k;
            hi[o] = h;
            lo[o] = l;
        }
    }
}

// R (float4 per sequence) -> B rows p*4+a, columns i, fp16 hi and lo of R*2^e
__global__ void k_split_R(const int32_t *__restrict__ list, int64_t Nx, const float4 *__restrict__ R, float sc,
                          __half *__restrict__ hi, __half *__restrict__ lo, int direct)
{
    const int P = blockIdx.y;
    const int b = direct ? P : list[P];   // direct: R rows by list position (digit planes)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < Nx; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = R[(int64_t)b * Nx + i];
        const float vv[4] = {v.x * sc, v.y * sc, v.z * sc, v.w * sc};
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const __half h = __float2half_rn(vv[a]);
            const __half l = __float2half_rn(vv[a] - __half2float(h));
            const int64_t o = ((int64_t)P * 4 + a) * Nx + i;
            hi[o] = h;
            lo[o] = l;
        }
    }
}

} // namespace tc

// ---------------------------------------------------------------------------
// host side

namespace {

using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn()
{
    // initialised once, thread-safely (solver lanes create plans concurrently)
    static const EncodeFn fn = []() -> EncodeFn {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeFn>(p);
        return nullptr;
    }();
    return fn;
}

bool make_map(CUtensorMap *m, CUtensorMapDataType dt, void *base, uint64_t cols, uint64_t rows,
              uint64_t row_bytes, uint32_t box_cols, uint32_t box_rows, CUtensorMapSwizzle sw)
{
    EncodeFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {row_bytes};
    const cuuint32_t box[2] = {box_cols, box_rows};
    const cuuint32_t es[2] = {1, 1};
    return fn(m, dt, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

} // namespace

struct TcPlan {
    CUtensorMap mX, mXT, mDhi, mDlo, mRhi, mRlo;
    bool has_fwd = false;   // the forward's slot operand (null for the dual form, which has no forward GEMM)
    int64_t Kp = 0;
    int fwd_splits = 1;
};

namespace {

// Subtiles per CTA (MSUB) and pipeline depth: {4, 2} keeps four 128-row
// accumulators (all 512 TMEM columns) and two 104 KB stages; {2, 3} and
// {1, 4} trade L2 reuse of the slot operand for deeper pipelines.
// SDCA_TC_MSUB (1, 2 or 4) overrides the choice for tuning runs.
int msub_choice()
{
    static const int v = []() {
        const char *e = std::getenv("SDCA_TC_MSUB");
        return (e && (e[0] == '1' || e[0] == '2')) ? e[0] - '0' : 4;
    }();
    return v;
}

template <int MSUB, int STG, int NT = 1, bool AT = false>
void launch_gemm(dim3 grid, const CUtensorMap &a, const CUtensorMap &bh, const CUtensorMap &bl,
                 const tc::GemmArgs &args, cudaStream_t st)
{
    tc::k_gemm<MSUB, STG, NT, AT>
        <<<grid, tc::THREADS, tc::Cfg<MSUB, STG, NT, AT>::SMEM_BYTES, st>>>(a, bh, bl, args);
}

// The backward with hi + lo operands (the tensor-core form's gradient, the
// dual form's max-norm checks) keeps its one-hot A in TMEM: two subtiles,
// four stages of 36 KB, the MMAs' N fitted to the live columns.  Measured
// with ncu on the 3000 x 94,000 workload (192-slot check launches): 337-375
// against 426-439 us for A in shared memory.  Exact (hi-only) operands -- the
// dual form's solution digit planes, two N tiles per CTA -- stay with A in
// shared memory: the TMEM form with one subtile and six stages took 689
// against 607 us there.  SDCA_TC_BWD_SMEM_A=1 keeps A in shared memory
// everywhere.
bool bwd_tmem_a()
{
    static const bool v = [] {
        const char *e = std::getenv("SDCA_TC_BWD_SMEM_A");
        return !(e && e[0] == '1');
    }();
    return v;
}

void launch_gemm_any(int msub, int m_tiles, int n_tiles, int splits, const CUtensorMap &a, const CUtensorMap &bh,
                     const CUtensorMap &bl, const tc::GemmArgs &args, cudaStream_t st)
{
    if (args.mode == tc::MODE_BWD && !args.hi_only && bwd_tmem_a()) {
        const dim3 grid((unsigned)((m_tiles + 1) / 2), (unsigned)n_tiles, (unsigned)splits);
        launch_gemm<2, 4, 1, true>(grid, a, bh, bl, args, st);
        return;
    }
    if (args.hi_only && args.mode == tc::MODE_BWD) {
        // exact fp16 operands: two N tiles per CTA, two subtiles, three stages
        const dim3 grid((unsigned)((m_tiles + 1) / 2), (unsigned)((n_tiles + 1) / 2), (unsigned)splits);
        launch_gemm<2, 3, 2>(grid, a, bh, bl, args, st);
        return;
    }
    const dim3 grid((unsigned)((m_tiles + msub - 1) / msub), (unsigned)n_tiles, (unsigned)splits);
    if (msub == 4) launch_gemm<4, 2>(grid, a, bh, bl, args, st);
    else if (msub == 2) launch_gemm<2, 3>(grid, a, bh, bl, args, st);
    else launch_gemm<1, 4>(grid, a, bh, bl, args, st);
}

} // namespace

int tc_fwd_splits(const Problem &P, int nlist)
{
    // split K so that the CTAs fill whole waves of 152 SMs (one CTA per SM)
    const int msub = msub_choice();
    const int mt = (int)((P.Nx + tc::BM - 1) / tc::BM);
    const int mg = (mt + msub - 1) / msub;
    const int nt = (4 * nlist + tc::BN - 1) / tc::BN;
    const int kt = (int)((4 * P.L + tc::BK - 1) / tc::BK);
    int best = 1;
    double best_t = 1e30;
    for (int s = 1; s <= (int)P.C; ++s) {
        const double waves = std::ceil((double)mg * nt * s / 152.0);
        const double t = waves * std::ceil((double)kt / s) + 8.0 * waves;
        if (t < best_t) {
            best_t = t;
            best = s;
        }
    }
    // no empty split: every launched split owns at least one k-tile
    const int stride = (kt + best - 1) / best;
    return (kt + stride - 1) / stride;
}

TcPlan *tc_plan_create(const Problem &P, const uint8_t *X, const uint8_t *XT, __half *Dhi, __half *Dlo,
                       __half *Rhi, __half *Rlo, int64_t Kp)
{
    TcPlan *p = new TcPlan();
    p->Kp = Kp;
    bool ok = true;
    ok &= make_map(&p->mX, CU_TENSOR_MAP_DATA_TYPE_UINT8, const_cast<uint8_t *>(X), (uint64_t)P.Lx,
                   (uint64_t)P.N, (uint64_t)P.Lx, 16, 128, CU_TENSOR_MAP_SWIZZLE_NONE);
    ok &= make_map(&p->mXT, CU_TENSOR_MAP_DATA_TYPE_UINT8, const_cast<uint8_t *>(XT), (uint64_t)P.Nx,
                   (uint64_t)P.L, (uint64_t)P.Nx, 64, 32, CU_TENSOR_MAP_SWIZZLE_NONE);
    p->has_fwd = Dhi && Dlo;
    if (p->has_fwd) {
        ok &= make_map(&p->mDhi, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, Dhi, (uint64_t)Kp, (uint64_t)4 * P.Bmax,
                       (uint64_t)Kp * 2, 64, 128, CU_TENSOR_MAP_SWIZZLE_128B);
        ok &= make_map(&p->mDlo, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, Dlo, (uint64_t)Kp, (uint64_t)4 * P.Bmax,
                       (uint64_t)Kp * 2, 64, 128, CU_TENSOR_MAP_SWIZZLE_128B);
    }
    ok &= make_map(&p->mRhi, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, Rhi, (uint64_t)P.Nx, (uint64_t)4 * P.Bmax,
                   (uint64_t)P.Nx * 2, 64, 128, CU_TENSOR_MAP_SWIZZLE_128B);
    ok &= make_map(&p->mRlo, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, Rlo, (uint64_t)P.Nx, (uint64_t)4 * P.Bmax,
                   (uint64_t)P.Nx * 2, 64, 128, CU_TENSOR_MAP_SWIZZLE_128B);
    if (!ok) {
        delete p;
        return nullptr;
    }
    return p;
}

void tc_plan_destroy(TcPlan *p) { delete p; }

struct KdPlan {
    CUtensorMap mK, mRh, mRt;   // K digits; rho digit plane heads (32 rows) and tails (8 rows)
    int nk_rows = 0, nr_rows = 0;
};

int kd_nk_rows(const Problem &P) { return (int)(((P.Nx + tc::KD_BM - 1) / tc::KD_BM) * tc::KD_BM); }
// rows per rho digit plane: 3 per slot for whole CTAs of 13 slots, one more
// for the last CTA's unused row, rounded to 8
int kd_nr_rows(const Problem &P)
{
    const int64_t slots = (P.Bmax + tc::KD_S - 1) / tc::KD_S * tc::KD_S;
    return (int)((tc::KD_C * slots + 1 + 7) / 8 * 8);
}

KdPlan *tc_kdig_plan_create(const Problem &P, __half *Kd, __half *Rd)
{
    KdPlan *p = new KdPlan();
    p->nk_rows = kd_nk_rows(P);
    p->nr_rows = kd_nr_rows(P);
    bool ok = make_map(&p->mK, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, Kd, (uint64_t)P.Nx, (uint64_t)tc::KD_KDIG * p->nk_rows,
                       (uint64_t)P.Nx * 2, tc::KD_BK, tc::KD_BM, CU_TENSOR_MAP_SWIZZLE_128B);
    ok &= make_map(&p->mRh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, Rd, (uint64_t)P.Nx, (uint64_t)tc::KD_RDIG * p->nr_rows,
                   (uint64_t)P.Nx * 2, tc::KD_BK, tc::KD_HEAD, CU_TENSOR_MAP_SWIZZLE_128B);
    if (tc::KD_TAIL > 0)
        ok &= make_map(&p->mRt, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, Rd, (uint64_t)P.Nx, (uint64_t)tc::KD_RDIG * p->nr_rows,
                       (uint64_t)P.Nx * 2, tc::KD_BK, tc::KD_TAIL > 0 ? tc::KD_TAIL : 8, CU_TENSOR_MAP_SWIZZLE_128B);
    if (!ok) {
        delete p;
        return nullptr;
    }
    return p;
}

void tc_kdig_plan_destroy(KdPlan *p) { delete p; }

void tc_kdig_fill_k(const KdPlan *pl, const Problem &P, const int32_t *K, __half *Kd, cudaStream_t st)
{
    const int64_t total = (int64_t)pl->nk_rows * P.Nx;
    tc::k_kdig_split_k<<<(unsigned)std::min<int64_t>((total + 255) / 256, 8192), 256, 0, st>>>(K, P.Nx, pl->nk_rows,
                                                                                          Kd);
}

cudaError_t tc_launch_kdig(const KdPlan *pl, const Problem &P, const int32_t *list, int n, const int32_t *rq,
                           const uint8_t *rstate, const long long *csum, double inv_qscale, __half *Rd, float2 *KR,
                           int *err, cudaStream_t st, const int *cnt)
{
    if (n <= 0) return cudaSuccess;
    {
        dim3 g((unsigned)std::min<int64_t>((P.Nx + 255) / 256, 64), (unsigned)n);
        tc::k_kdig_split_r<<<g, 256, 0, st>>>(list, P.Nx, pl->nr_rows, reinterpret_cast<const int4 *>(rq), Rd, cnt);
    }
    tc::KdArgs a{};
    a.kt_total = (int)(P.Nx / tc::KD_BK);
    a.nk_rows = pl->nk_rows;
    a.nr_rows = pl->nr_rows;
    a.N = (int)P.N;
    a.Nx = P.Nx;
    a.nlist = n;
    a.list = list;
    a.rstate = rstate;
    a.csum = csum;
    a.inv_qscale = inv_qscale;
    a.KR = KR;
    a.err = err;
    a.ncount = cnt;
    dim3 grid((unsigned)(pl->nk_rows / tc::KD_BM), (unsigned)((n + tc::KD_S - 1) / tc::KD_S));
    tc::k_kdig<<<grid, tc::THREADS, tc::KD_SMEM, st>>>(pl->mK, pl->mRh, pl->mRt, a);
    return cudaGetLastError();
}

cudaError_t tc_launch_fwd(const TcPlan *pl, const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                          const float *vecs, __half *Dhi, __half *Dlo, float *partial, int splits, int *err,
                          cudaStream_t st)
{
    if (!pl->has_fwd) return cudaErrorInvalidValue;   // a plan without the forward's operand
    if (n <= 0) return cudaSuccess;
    {
        dim3 g((unsigned)std::min<int64_t>((4 * P.L + 255) / 256, 1024), (unsigned)n);
        tc::k_split_dir<<<g, 256, 0, st>>>(sd, list, P.L, P.Dp, pl->Kp, vecs, Dhi, Dlo);
    }
    tc::GemmArgs a{};
    a.mode = tc::MODE_FWD;
    a.kt_total = (int)((4 * P.L + tc::BK - 1) / tc::BK);
    a.kt_begin_stride = (a.kt_total + splits - 1) / splits;
    a.m_rows = (int)P.N;
    a.nlist = n;
    a.list = list;
    a.sd = sd;
    a.partial = reinterpret_cast<float4 *>(partial);
    a.Bmax = P.Bmax;
    a.Nx = P.Nx;
    a.err = err;
    launch_gemm_any(msub_choice(), (int)((P.Nx + tc::BM - 1) / tc::BM), (4 * n + tc::BN - 1) / tc::BN, splits,
                    pl->mX, pl->mDhi, pl->mDlo, a, st);
    return cudaGetLastError();
}

cudaError_t tc_launch_bwd(const TcPlan *pl, const Problem &P, const SlotDev *sd, const int32_t *list, int n,
                          const float *R, float r_scale, __half *Rhi, __half *Rlo, float *gpool, int *err,
                          cudaStream_t st, bool exact_fp16, double *gmax_acc, int gmax_stride, int planes)
{
    if (n <= 0) return cudaSuccess;
    const int nslot = n;
    if (planes > 1) {
        if ((int64_t)planes * n > P.Bmax) return cudaErrorInvalidValue;   // B operand rows and gpool buffers
        n *= planes;
    }
    {
        dim3 g((unsigned)std::min<int64_t>((P.Nx + 255) / 256, 64), (unsigned)n);
        tc::k_split_R<<<g, 256, 0, st>>>(list, P.Nx, reinterpret_cast<const float4 *>(R), r_scale, Rhi, Rlo,
                                          planes > 1 ? 1 : 0);
    }
    tc::GemmArgs a{};
    a.mode = tc::MODE_BWD;
    a.kt_total = (int)(P.Nx / tc::BK);
    a.kt_begin_stride = a.kt_total;
    a.m_rows = (int)(4 * P.L);
    a.nlist = n;
    a.list = list;
    a.sd = sd;
    a.gpool = gpool;
    a.Dp = P.Dp;
    a.inv_scale_bwd = 1.0f / r_scale;
    a.hi_only = exact_fp16 ? 1 : 0;
    a.gmax_acc = gmax_acc;
    a.gmax_stride = gmax_stride;
    a.planes = planes > 1 ? planes : 1;
    a.nslot = nslot;
    a.Nx = P.Nx;
    a.err = err;
    launch_gemm_any(msub_choice(), (int)((4 * P.L + tc::BM - 1) / tc::BM), (4 * n + tc::BN - 1) / tc::BN, 1,
                    pl->mXT, pl->mRhi, pl->mRlo, a, st);
    return cudaGetLastError();
}

cudaError_t tc_configure()
{
    cudaError_t e = cudaFuncSetAttribute(tc::k_gemm<4, 2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::Cfg<4, 2>::SMEM_BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tc::k_gemm<2, 3, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc::Cfg<2, 3, 2>::SMEM_BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tc::k_gemm<2, 3, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc::Cfg<2, 3>::SMEM_BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tc::k_gemm<1, 4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc::Cfg<1, 4>::SMEM_BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tc::k_gemm<2, 4, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc::Cfg<2, 4, 1, true>::SMEM_BYTES);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tc::k_kdig, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::KD_SMEM);
    return e;
}

} // namespace sdca

// Mixed-precision perturbation averages on the 5th-generation tensor cores.
//
// Same GEMM form as the float64 path (perturb_fp64.cu):
//   stage A   V = D Y1           (R x M x M)   -> per-row q, p, s, t in the epilogue
//   stage B   G = U^T W          (M x M x R)   -> split-K fp32 partial tiles
// Every operand row of the K-major layout is scaled into [-1, 1] by a per-mode
// (or per-row) factor and held as two fp16 limbs,
//   x = hi + lo * 2^-11,   hi = fp16(x),   lo = fp16((x - hi) * 2^11),
// about 22 significant bits; the low limb is kept at the magnitude of the high
// one so it never falls into the fp16 subnormal range.  Each product is
// hi*hi into TMEM accumulator D0 and hi*lo + lo*hi into accumulator D1 (three
// tcgen05.mma per K step); the epilogue forms D0 + 2^-11 D1 and undoes the
// scales.  The Lanczos recurrence around it stays in float64.
//
// Scales: stage A multiplies the K (mode) axis by 1/sd_m on D and by sd_m on
// Y1 (sd_m = max_r |D[r][m]|, fixed per ensemble), and each Y1 row n by 1/t_n
// (its max, per call); stage B scales U^T row a by 1/su_a (su_a = f_Y,a sd_a)
// and W^T row b by 1/sw_b, an upper bound of max_r |W[r][b]| from the maxima
// of alpha, beta, F and U.
//
// Kernel anatomy (k_stageA_tc, k_stageB_tc): persistent, one CTA per SM,
// 192 threads, accumulators double-buffered in TMEM.
//   warp 4 lane 0  TMA producer: cp.async.bulk.tensor 2D loads of the four
//                  operand tiles (A hi/lo 128x64, B hi/lo 128x64, 128B swizzle)
//                  into a 3-stage ring, completion on mbarrier full[s]
//   warp 5 lane 0  MMA issuer: 4 K-slices x 3 products per stage, then
//                  tcgen05.commit -> empty[s]; per tile a commit -> tfull[j]
//   warps 0-3      epilogue: tcgen05.ld 32x32b (warp w owns TMEM lanes
//                  32w..32w+31) from TMEM half j while the next tile's MMAs
//                  fill the other half; fused row dots (A) or tile store (B)
// Every mbarrier wait is bounded (clock64 budget); on expiry the kernel sets
// the context's error flag and a shared abort flag that ends the other roles'
// loops, drains its own copies and MMAs (bounded again), frees its TMEM and
// returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "dfloat.cuh"

namespace tdscha {

constexpr int kBM = 128;          // tile rows (TMEM lanes)
constexpr int kBK = 64;           // K block: 64 fp16 = one 128-byte swizzle row
constexpr uint32_t kABytes = kBM * kBK * 2;
constexpr int kBNB = 128;         // stage B tile width
// stage B rows per split: the length of one fp32 accumulation in TMEM.  1024
// rather than 2048 halves the spectral error of a 300-step run at M=573,
// N=50 000 on four of five seeded ensembles (e.g. 8.97e-5 -> 4.53e-5) for 3 %
// more run time (more partial tiles to sum).
constexpr int kSplitRows = 1024;
constexpr float kLoScale = 2048.f;
constexpr float kLoInv = 1.f / 2048.f;
constexpr long long kDefaultBudget = 4000000000LL;   // ~2 s at 2 GHz

struct TmaQuad {
    CUtensorMap a_hi, a_lo, b_hi, b_lo;
};

// fp32 row tiles read by the stage A epilogue (d and g = f_psi * f)
struct TmaEpi {
    CUtensorMap d, g;
};


// ------------------------------------------------------------------ PTX
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase of the given parity; false when the budget runs out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long budget) {
    long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (clock64() - t0 > budget) return false;
    }
    return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, uint32_t bar,
                                            int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand in the 128-byte swizzle
// layout written by TMA (8-row groups 1024 bytes apart).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);          // start address
    d |= (uint64_t)(16 >> 4) << 16;                 // leading byte offset (unused for SW128 K-major)
    d |= (uint64_t)(1024 >> 4) << 32;               // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                         // descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;                         // layout: 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: A = B = fp16, D = f32, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
    return (1u << 4)                      // D format f32 (A, B format fields 0 = fp16)
           | ((uint32_t)(N >> 3) << 17)   // N / 8
           | ((uint32_t)(M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
          "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
          "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
          "=r"(v[31])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int NCOLS>
__device__ __forceinline__ void tmem_alloc(uint32_t slot) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
                 "n"(NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

template <int NCOLS>
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "n"(NCOLS)
                 : "memory");
}

// D0 + 2^-11 D1 for 32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_combined(uint32_t lane_base, int col, int bn, float (&o)[32]) {
    uint32_t v0[32], v1[32];
    tmem_ld32(lane_base + col, v0);
    tmem_ld32(lane_base + bn + col, v1);
    tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 32; ++j) o[j] = fmaf(__uint_as_float(v1[j]), kLoInv, __uint_as_float(v0[j]));
}

// ------------------------------------------------- persistent stage A
// One CTA per SM walks a contiguous range of the 128 x 128 tiles of V = D Y1
// (row tile major, column tile minor): the first column tile of a row block
// pulls its A rows from HBM and the others re-read them from L2, while the
// SMs work on row blocks far apart (no two SMs waiting on the same misses).
// Warp roles:
//   warps 0-3  epilogue: warp w owns TMEM lanes (tile rows) 32w..32w+31
//   warp 4     TMA producer of the operand ring
//   warp 5     MMA issuer (and TMEM owner)
// D0 / D1 of a tile take 2 x 128 TMEM columns; two tiles' accumulators are
// resident (512 columns), so the epilogue of tile i (TMEM reads and the
// q, p, s, t row dots) runs while the MMAs of tile i+1 fill the other half.
// The epilogue's d and g rows come in by TMA in 16-column parts (64-byte
// swizzle) through a two-part ring that its leader thread keeps two parts
// ahead, across tiles; that keeps the operand ring at three 64 KB stages.
// Every wait is bounded; a failed wait sets the error flag and a shared
// abort flag that ends the other roles' loops, in-flight copies and MMAs are
// drained (bounded again) and the TMEM is freed before the CTA exits.
constexpr int kPBN = 128;                                   // tile columns
constexpr int kPBK = kBK;                                   // K block: one 128-byte swizzle row
constexpr int kPStages = 3;
constexpr uint32_t kPLimbA = kBM * kPBK * 2;                // 16 KB
constexpr uint32_t kPLimbB = kPBN * kPBK * 2;               // 16 KB
constexpr uint32_t kPStageBytes = 2 * kPLimbA + 2 * kPLimbB;   // 64 KB
constexpr int kPEpiCols = 16;                               // columns per epilogue part
constexpr uint32_t kPEpiBox = kBM * kPEpiCols * 4;          // 128 rows x 16 fp32
constexpr uint32_t kPEpiBytes = 2 * kPEpiBox;               // d and g of one part
constexpr int kPBars = 2 * kPStages + 7;                    // full, empty, tfull[2], tempty[2], efull[2], done
constexpr size_t kPSmem = 1024 + kPStages * (size_t)kPStageBytes + 2 * (size_t)kPEpiBytes +
                          3 * kPBN * sizeof(float) + 8 * kPBars + 16;
static_assert(kPSmem <= 232448, "stage A shared memory above the per-block limit");

struct StageAArgs {
    long R;               // rows of D
    int Mp;
    int nkb;              // k-blocks per tile (Mp / 64)
    int nct;              // column tiles per perturbation image (ceil(Mp / 128))
    int J;                // perturbation images: B = [Y1_0 ... Y1_{J-1}] (J x Mp rows)
    int b_box;            // rows of one B (Y1) box: min(128, Mp)
    long ntiles;
    const float *tcol, *vec_s, *vec_t;
    float *qpst;          // [J][nct][4][R]
    int *err;
    long long budget;
};

// Bounded wait that also gives up once another role has raised `abort`.
__device__ __forceinline__ bool mbar_wait_ab(uint32_t bar, uint32_t parity, long long budget,
                                             volatile int *abort) {
    long long t0 = clock64();
    uint32_t spins = 0;
    while (!mbar_try(bar, parity)) {
        if ((++spins & 31u) == 0 && *abort) return false;
        if (clock64() - t0 > budget) return false;
    }
    return true;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Named barrier 1 over the 128 epilogue threads; returns true if `pred` was
// set in any of them.
__device__ __forceinline__ bool epi_sync_or(bool pred) {
    uint32_t out;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, 1, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(out)
        : "r"((uint32_t)pred)
        : "memory");
    return out != 0;
}

__global__ void __launch_bounds__(192, 1) k_stageA_tc(const __grid_constant__ TmaQuad tm,
                                                       const __grid_constant__ TmaEpi te,
                                                       const StageAArgs args) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *epi = smem + kPStages * kPStageBytes;
    float *colv = reinterpret_cast<float *>(epi + 2 * kPEpiBytes);   // [3][kPBN]
    uint64_t *bars = reinterpret_cast<uint64_t *>(colv + 3 * kPBN);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + kPBars);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * kPStages,
                   tfull0 = empty0 + 8 * kPStages, tempty0 = tfull0 + 16, efull0 = tempty0 + 16,
                   done = efull0 + 16;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long budget = args.budget;
    const long G = gridDim.x;
    // this CTA's tiles: [t0, t0 + nloc), an even split of the tile sequence
    const long t0 = args.ntiles * blockIdx.x / G;
    const long nloc = args.ntiles * (blockIdx.x + 1) / G - t0;
    const int nct = args.nct, Mp = args.Mp;
    const long jn = (long)args.J * nct;   // tiles per row block: images x column tiles
    const uint32_t b_bytes = (uint32_t)args.b_box * kPBK * 2;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kPStages; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int j = 0; j < 2; ++j) {
            mbar_init(tfull0 + 8 * j, 1);
            mbar_init(tempty0 + 8 * j, 128);
            mbar_init(efull0 + 8 * j, 1);
        }
        mbar_init(done, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 5) tmem_alloc<512>(smem_u32(tmem_slot));
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // barriers and TMEM are set up; global memory only after the kernels
    // before this one in the stream have completed
    pdl_enter();
    int fail_code = 0;

    if (warp == 4) {
        if (lane == 0) {
            // ---- TMA producer: the operand ring, continuous across tiles
            long g = 0;
            for (long i = 0; i < nloc && !fail_code; ++i) {
                long t = t0 + i;
                const long rem = t % jn;
                int arow = (int)(t / jn) * kBM;
                int brow = (int)(rem / nct) * Mp + (int)(rem % nct) * kPBN;   // row of Y1_j
                for (int kb = 0; kb < args.nkb; ++kb, ++g) {
                    int s = (int)(g % kPStages);
                    uint32_t n = (uint32_t)(g / kPStages);
                    if (g >= kPStages && !mbar_wait_ab(empty0 + 8 * s, (n & 1) ^ 1, budget, abort)) {
                        fail_code = 1;
                        break;
                    }
                    uint32_t base = smem_u32(smem + s * kPStageBytes);
                    uint32_t bar = full0 + 8 * s;
                    int kx = kb * kPBK;
                    mbar_expect_tx(bar, 2 * kPLimbA + 2 * b_bytes);
                    tma_load_2d(base, &tm.a_hi, bar, kx, arow);
                    tma_load_2d(base + kPLimbA, &tm.a_lo, bar, kx, arow);
                    tma_load_2d(base + 2 * kPLimbA, &tm.b_hi, bar, kx, brow);
                    tma_load_2d(base + 2 * kPLimbA + kPLimbB, &tm.b_lo, bar, kx, brow);
                }
            }
            if (fail_code) {
                *abort = 1;
                // every issued stage must land before the CTA exits
                for (long gg = g > kPStages ? g - kPStages : 0; gg < g; ++gg)
                    mbar_wait(full0 + 8 * (int)(gg % kPStages), (uint32_t)(gg / kPStages) & 1,
                              kDefaultBudget);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            // ---- MMA issuer: D0 += hi*hi, D1 += hi*lo + lo*hi, tile i into
            // TMEM half (i & 1)
            long g = 0;
            for (long i = 0; i < nloc && !fail_code; ++i) {
                long t = t0 + i;
                int brow = (int)((t % jn) % nct) * kPBN;
                int ncols = min(kPBN, Mp - brow);
                const uint32_t idesc = idesc_f16(kBM, ncols);
                int j = (int)(i & 1);
                uint32_t u = (uint32_t)(i >> 1);
                if (i >= 2 && !mbar_wait_ab(tempty0 + 8 * j, (u - 1) & 1, budget, abort)) {
                    fail_code = 2;
                    break;
                }
                tc_fence_after();
                const uint32_t d0 = tmem + 256 * j, d1 = d0 + 128;
                for (int kb = 0; kb < args.nkb; ++kb, ++g) {
                    int s = (int)(g % kPStages);
                    uint32_t n = (uint32_t)(g / kPStages);
                    if (!mbar_wait_ab(full0 + 8 * s, n & 1, budget, abort)) {
                        fail_code = 2;
                        break;
                    }
                    tc_fence_after();
                    uint32_t base = smem_u32(smem + s * kPStageBytes);
#pragma unroll
                    for (int kk = 0; kk < kPBK / 16; ++kk) {
                        uint64_t ah = sdesc_sw128(base + kk * 32);
                        uint64_t al = sdesc_sw128(base + kPLimbA + kk * 32);
                        uint64_t bh = sdesc_sw128(base + 2 * kPLimbA + kk * 32);
                        uint64_t bl = sdesc_sw128(base + 2 * kPLimbA + kPLimbB + kk * 32);
                        uint32_t acc = (kb | kk) != 0;
                        mma_f16(d0, ah, bh, idesc, acc);
                        mma_f16(d1, ah, bl, idesc, acc);
                        mma_f16(d1, al, bh, idesc, 1);
                    }
                    mma_commit(empty0 + 8 * s);
                }
                if (fail_code) break;
                mma_commit(tfull0 + 8 * j);
            }
            if (fail_code) *abort = 1;
            mma_commit(done);   // tracks every MMA issued, also after a failure
        }
    } else {
        // ---- epilogue (warps 0-3): thread = tile row = TMEM lane
        const int row_in = warp * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        const bool leader = threadIdx.x == 0;
        // leader's cursor over the (tile, part) sequence of epilogue loads
        long iss_i = 0, issued = 0;
        int iss_p = 0;
        auto issue_next = [&]() {
            if (iss_i >= nloc) return;
            long t = t0 + iss_i;
            int arow = (int)(t / jn) * kBM, brow = (int)((t % jn) % nct) * kPBN;
            int e = (int)(issued & 1);
            uint32_t buf = smem_u32(epi + e * kPEpiBytes), bar = efull0 + 8 * e;
            int x = brow + iss_p * kPEpiCols;
            mbar_expect_tx(bar, kPEpiBytes);
            tma_load_2d(buf, &te.d, bar, x, arow);
            tma_load_2d(buf + kPEpiBox, &te.g, bar, x, arow);
            ++issued;
            if (++iss_p == min(kPBN, Mp - brow) / kPEpiCols) {
                iss_p = 0;
                ++iss_i;
            }
        };
        if (leader) {
            issue_next();
            issue_next();
        }
        long consumed = 0;
        for (long i = 0; i < nloc; ++i) {
            long t = t0 + i;
            const int jimg = (int)((t % jn) / nct);
            const int ct = (int)((t % jn) % nct);
            const int brow = ct * kPBN;
            const long row = (long)(t / jn) * kBM + row_in;
            const int np = min(kPBN, Mp - brow) / 32;   // 32-column TMEM chunks
            const int j = (int)(i & 1);
            const uint32_t u = (uint32_t)(i >> 1);
            // column factors of this tile; the previous tile's last reads of
            // them came before its last part barrier
            float *cv = colv;
            {
                int c = brow + row_in;
                bool in = c < Mp;
                long cj = (long)jimg * Mp + c;
                cv[row_in] = in ? args.tcol[cj] : 0.f;
                cv[kPBN + row_in] = in ? args.vec_s[cj] : 0.f;
                cv[2 * kPBN + row_in] = in ? args.vec_t[cj] : 0.f;
            }
            bool ok = mbar_wait_ab(tfull0 + 8 * j, u & 1, budget, abort);
            __syncwarp();
            if (epi_sync_or(!ok)) {   // also publishes cv to the other warps
                fail_code = 3;
                break;
            }
            tc_fence_after();
            float q = 0.f, p = 0.f, sacc = 0.f, tacc = 0.f;
            for (int chunk = 0; chunk < np; ++chunk) {
                float v[32];
                tmem_combined(lane_base + 256 * j, chunk * 32, 128, v);
                if (chunk == np - 1) {
                    // this tile's accumulators are read: release the TMEM half
                    tc_fence_before();
                    mbar_arrive(tempty0 + 8 * j);
                }
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    const int e = (int)(consumed & 1);
                    bool landed = mbar_wait_ab(efull0 + 8 * e, (uint32_t)(consumed >> 1) & 1,
                                               budget, abort);
                    __syncwarp();
                    if (epi_sync_or(!landed)) {
                        fail_code = 3;
                        break;
                    }
                    // 64-byte rows, 16-byte granule c stored at c ^ ((row >> 1) & 3)
                    const uint8_t *bd = epi + e * kPEpiBytes + row_in * 64;
                    const uint8_t *bg = bd + kPEpiBox;
                    const int sw = (row_in >> 1) & 3;
                    const float *cp = cv + chunk * 32 + half * 16;
#pragma unroll
                    for (int ch = 0; ch < 4; ++ch) {
                        float4 d4 = *reinterpret_cast<const float4 *>(bd + ((ch ^ sw) << 4));
                        float4 g4 = *reinterpret_cast<const float4 *>(bg + ((ch ^ sw) << 4));
                        float dd[4] = {d4.x, d4.y, d4.z, d4.w}, gg[4] = {g4.x, g4.y, g4.z, g4.w};
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            int c = 4 * ch + k;
                            float vv = v[half * 16 + c] * cp[c];
                            q = fmaf(dd[k], vv, q);
                            p = fmaf(gg[k], vv, p);
                            sacc = fmaf(cp[kPBN + c], dd[k], sacc);
                            tacc = fmaf(cp[2 * kPBN + c], gg[k], tacc);
                        }
                    }
                    ++consumed;
                    // every epilogue thread is done with buffer e: refill it.
                    // The reads above are generic-proxy and the refill is a TMA
                    // write (async proxy); the barrier alone does not order the
                    // two, and a refill that landed before a slow warp's loads
                    // had read the part gave wrong d values in a few rows of one
                    // tile in about one call in 1500 (M=573, N=20 000)
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("bar.sync 1, 128;" ::: "memory");
                    if (leader) issue_next();
                }
                if (fail_code) break;
            }
            if (fail_code) break;
            if (row < args.R) {
                const long R = args.R;
                float *o = args.qpst + ((long)jimg * nct + ct) * 4 * R;
                o[row] = q;
                o[R + row] = p;
                o[2 * R + row] = sacc;
                o[3 * R + row] = tacc;
            }
        }
        if (fail_code) {
            *abort = 1;
            if (leader)
                for (long k = consumed; k < issued; ++k)
                    mbar_wait(efull0 + 8 * (int)(k & 1), (uint32_t)(k >> 1) & 1, kDefaultBudget);
        }
    }
    if (fail_code && lane == 0) *(volatile int *)args.err = fail_code;
    tc_fence_before();
    __syncthreads();
    if (warp == 5) {
        // every MMA has completed before the TMEM is freed
        mbar_wait(done, 0, kDefaultBudget);
        __syncwarp();
        tc_fence_after();
        tmem_dealloc<512>(tmem);
    }
}

// ------------------------------ stage A with one accumulator per tile
// The same product as k_stageA_tc (tiles of V = D [Y1_0 ... Y1_{J-1}], fused
// row dots) with 128 x 192 tiles, so that a whole 189-mode image or a third
// of 573 modes is one N=192 MMA.  The hi*lo + lo*hi products of a tile are
// accumulated first over the whole K range; the first hi*hi MMA then scales
// the accumulator by 2^-11 on the way in (tcgen05.mma's scale-input-d), and
// the rest of the hi*hi products follow, so D = sum hi*hi + 2^-11 sum
// (hi*lo + lo*hi) sits in one fp32 accumulator (192 TMEM columns) and two
// tiles' accumulators fit in the 512 columns (double buffering).  The
// operands pass through the ring twice per tile (the hi limbs twice), in
// 40 KB slots: [A limb 128 x 64 | B limb 192 x 64].
constexpr int kRBN = 192;
constexpr int kRSlots = 4;
constexpr uint32_t kRLimbA = kBM * kBK * 2;                  // 16 KB
constexpr uint32_t kRSlotBytes = kRLimbA + kRBN * kBK * 2;   // 40 KB
// epilogue part buffers (d and g parts, one TMA load each from L2).  Three
// buffers (two parts in flight while one is read) made this kernel slower at
// M = 189, 48 images: 273 us against 262 us per launch with two
constexpr int kREpiBufs = 2;
constexpr int kRBars = 2 * kRSlots + 5 + kREpiBufs;   // full, empty, tfull[2], tempty[2], efull[], done
constexpr size_t kRSmem = 1024 + kRSlots * (size_t)kRSlotBytes + kREpiBufs * (size_t)kPEpiBytes +
                          3 * kRBN * sizeof(float) + 8 * kRBars + 16;
static_assert(kRSmem <= 232448, "stage A (one accumulator) shared memory above the limit");

__device__ __forceinline__ void mma_f16_scaled11(uint32_t tmem, uint64_t a, uint64_t b,
                                                 uint32_t idesc) {
    // D = A B + D 2^-11
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, 1, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p, 11;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc)
        : "memory");
}

__global__ void __launch_bounds__(192, 1) k_stageA_tc1(const __grid_constant__ TmaQuad tm,
                                                       const __grid_constant__ TmaEpi te,
                                                       const StageAArgs args) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *epi = smem + kRSlots * kRSlotBytes;
    float *colv = reinterpret_cast<float *>(epi + kREpiBufs * kPEpiBytes);   // [3][kRBN]
    uint64_t *bars = reinterpret_cast<uint64_t *>(colv + 3 * kRBN);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + kRBars);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * kRSlots,
                   tfull0 = empty0 + 8 * kRSlots, tempty0 = tfull0 + 16, efull0 = tempty0 + 16,
                   done = efull0 + 8 * kREpiBufs;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long budget = args.budget;
    const long G = gridDim.x;
    // this CTA's tiles: [t0, t0 + nloc), an even split of the tile sequence
    const long t0 = args.ntiles * blockIdx.x / G;
    const long nloc = args.ntiles * (blockIdx.x + 1) / G - t0;
    const int nct = args.nct, Mp = args.Mp;
    const long jn = (long)args.J * nct;   // tiles per row block: images x column tiles
    const uint32_t b_bytes = (uint32_t)args.b_box * kBK * 2;
    const int nkb = args.nkb;
    const int slots_per_tile = 3 * nkb;   // cross pass: 2 slots per K block, hi pass: 1

    if (threadIdx.x == 0) {
        for (int s = 0; s < kRSlots; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int j = 0; j < 2; ++j) {
            mbar_init(tfull0 + 8 * j, 1);
            mbar_init(tempty0 + 8 * j, 128);
        }
        for (int j = 0; j < kREpiBufs; ++j) mbar_init(efull0 + 8 * j, 1);
        mbar_init(done, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 5) tmem_alloc<512>(smem_u32(tmem_slot));
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // barriers and TMEM are set up; global memory only after the kernels
    // before this one in the stream have completed
    pdl_enter();
    int fail_code = 0;

    if (warp == 4) {
        if (lane == 0) {
            // ---- TMA producer: per tile the cross pass (slot pairs (A hi, B lo),
            // (A lo, B hi) per K block), then the hi pass ((A hi, B hi) per K block)
            long g = 0;
            for (long i = 0; i < nloc && !fail_code; ++i) {
                long t = t0 + i;
                const long rem = t % jn;
                int arow = (int)(t / jn) * kBM;
                int brow = (int)(rem / nct) * Mp + (int)(rem % nct) * kRBN;   // row of Y1_j
                for (int q = 0; q < slots_per_tile; ++q, ++g) {
                    const bool cross = q < 2 * nkb;
                    const int kb = cross ? q >> 1 : q - 2 * nkb;
                    const bool second = cross && (q & 1);
                    int s = (int)(g % kRSlots);
                    uint32_t n = (uint32_t)(g / kRSlots);
                    if (g >= kRSlots && !mbar_wait_ab(empty0 + 8 * s, (n & 1) ^ 1, budget, abort)) {
                        fail_code = 1;
                        break;
                    }
                    uint32_t base = smem_u32(smem + s * kRSlotBytes);
                    uint32_t bar = full0 + 8 * s;
                    int kx = kb * kBK;
                    mbar_expect_tx(bar, kRLimbA + b_bytes);
                    tma_load_2d(base, second ? &tm.a_lo : &tm.a_hi, bar, kx, arow);
                    tma_load_2d(base + kRLimbA, (cross && !second) ? &tm.b_lo : &tm.b_hi, bar, kx,
                                brow);
                }
            }
            if (fail_code) {
                *abort = 1;
                // every issued slot must land before the CTA exits
                for (long gg = g > kRSlots ? g - kRSlots : 0; gg < g; ++gg)
                    mbar_wait(full0 + 8 * (int)(gg % kRSlots), (uint32_t)(gg / kRSlots) & 1,
                              kDefaultBudget);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            // ---- MMA issuer: one accumulator per tile, tile i in TMEM columns
            // 256 (i & 1): D = sum hi*lo + lo*hi over K, then D = hi*hi + D 2^-11
            // (the scale on the first hi*hi MMA), then D += hi*hi over K
            long g = 0;
            for (long i = 0; i < nloc && !fail_code; ++i) {
                long t = t0 + i;
                int brow = (int)((t % jn) % nct) * kRBN;
                int ncols = min(kRBN, Mp - brow);
                const uint32_t idesc = idesc_f16(kBM, ncols);
                int j = (int)(i & 1);
                uint32_t u = (uint32_t)(i >> 1);
                if (i >= 2 && !mbar_wait_ab(tempty0 + 8 * j, (u - 1) & 1, budget, abort)) {
                    fail_code = 2;
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + 256 * j;
                for (int q = 0; q < slots_per_tile && !fail_code;) {
                    const bool cross = q < 2 * nkb;
                    const int nsl = cross ? 2 : 1;
                    uint32_t base[2] = {0u, 0u};
                    for (int h = 0; h < nsl; ++h) {
                        int s = (int)((g + h) % kRSlots);
                        uint32_t n = (uint32_t)((g + h) / kRSlots);
                        if (!mbar_wait_ab(full0 + 8 * s, n & 1, budget, abort)) {
                            fail_code = 2;
                            break;
                        }
                        base[h] = smem_u32(smem + s * kRSlotBytes);
                    }
                    if (fail_code) break;
                    tc_fence_after();
                    const int kb = cross ? q >> 1 : q - 2 * nkb;
#pragma unroll
                    for (int kk = 0; kk < kBK / 16; ++kk) {
                        uint64_t a0 = sdesc_sw128(base[0] + kk * 32);
                        uint64_t b0 = sdesc_sw128(base[0] + kRLimbA + kk * 32);
                        if (cross) {
                            uint64_t a1 = sdesc_sw128(base[1] + kk * 32);
                            uint64_t b1 = sdesc_sw128(base[1] + kRLimbA + kk * 32);
                            mma_f16(d, a0, b0, idesc, (kb | kk) != 0);   // hi * lo
                            mma_f16(d, a1, b1, idesc, 1);                // lo * hi
                        } else if ((kb | kk) == 0) {
                            mma_f16_scaled11(d, a0, b0, idesc);          // hi * hi + D 2^-11
                        } else {
                            mma_f16(d, a0, b0, idesc, 1);
                        }
                    }
                    for (int h = 0; h < nsl; ++h) mma_commit(empty0 + 8 * (int)((g + h) % kRSlots));
                    g += nsl;
                    q += nsl;
                }
                if (fail_code) break;
                mma_commit(tfull0 + 8 * j);
            }
            if (fail_code) *abort = 1;
            mma_commit(done);   // tracks every MMA issued, also after a failure
        }
    } else {
        // ---- epilogue (warps 0-3): thread = tile row = TMEM lane
        const int row_in = warp * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        const bool leader = threadIdx.x == 0;
        // leader's cursor over the (tile, part) sequence of epilogue loads
        long iss_i = 0, issued = 0;
        int iss_p = 0;
        auto issue_next = [&]() {
            if (iss_i >= nloc) return;
            long t = t0 + iss_i;
            int arow = (int)(t / jn) * kBM, brow = (int)((t % jn) % nct) * kRBN;
            int e = (int)(issued % kREpiBufs);
            uint32_t buf = smem_u32(epi + e * kPEpiBytes), bar = efull0 + 8 * e;
            int x = brow + iss_p * kPEpiCols;
            mbar_expect_tx(bar, kPEpiBytes);
            tma_load_2d(buf, &te.d, bar, x, arow);
            tma_load_2d(buf + kPEpiBox, &te.g, bar, x, arow);
            ++issued;
            if (++iss_p == min(kRBN, Mp - brow) / kPEpiCols) {
                iss_p = 0;
                ++iss_i;
            }
        };
        if (leader)
            for (int b = 0; b < kREpiBufs; ++b) issue_next();
        long consumed = 0;
        for (long i = 0; i < nloc; ++i) {
            long t = t0 + i;
            const int jimg = (int)((t % jn) / nct);
            const int ct = (int)((t % jn) % nct);
            const int brow = ct * kRBN;
            const long row = (long)(t / jn) * kBM + row_in;
            const int np = min(kRBN, Mp - brow) / 32;   // 32-column TMEM chunks
            const int j = (int)(i & 1);
            const uint32_t u = (uint32_t)(i >> 1);
            // column factors of this tile; the previous tile's last reads of
            // them came before its last part barrier
            float *cv = colv;
            for (int cc = row_in; cc < kRBN; cc += kBM) {
                int c = brow + cc;
                bool in = c < Mp;
                long cj = (long)jimg * Mp + c;
                cv[cc] = in ? args.tcol[cj] : 0.f;
                cv[kRBN + cc] = in ? args.vec_s[cj] : 0.f;
                cv[2 * kRBN + cc] = in ? args.vec_t[cj] : 0.f;
            }
            bool ok = mbar_wait_ab(tfull0 + 8 * j, u & 1, budget, abort);
            __syncwarp();
            if (epi_sync_or(!ok)) {   // also publishes cv to the other warps
                fail_code = 3;
                break;
            }
            tc_fence_after();
            float q = 0.f, p = 0.f, sacc = 0.f, tacc = 0.f;
            for (int chunk = 0; chunk < np; ++chunk) {
                float v[32];
                {
                    uint32_t raw[32];
                    tmem_ld32(lane_base + 256 * j + chunk * 32, raw);
                    tmem_wait_ld();
#pragma unroll
                    for (int e = 0; e < 32; ++e) v[e] = __uint_as_float(raw[e]);
                }
                if (chunk == np - 1) {
                    // this tile's accumulators are read: release the TMEM half
                    tc_fence_before();
                    mbar_arrive(tempty0 + 8 * j);
                }
#pragma unroll
                for (int half = 0; half < 2; ++half) {
                    const int e = (int)(consumed % kREpiBufs);
                    bool landed = mbar_wait_ab(efull0 + 8 * e,
                                               (uint32_t)(consumed / kREpiBufs) & 1, budget, abort);
                    __syncwarp();
                    if (epi_sync_or(!landed)) {
                        fail_code = 3;
                        break;
                    }
                    // 64-byte rows, 16-byte granule c stored at c ^ ((row >> 1) & 3)
                    const uint8_t *bd = epi + e * kPEpiBytes + row_in * 64;
                    const uint8_t *bg = bd + kPEpiBox;
                    const int sw = (row_in >> 1) & 3;
                    const float *cp = cv + chunk * 32 + half * 16;
#pragma unroll
                    for (int ch = 0; ch < 4; ++ch) {
                        float4 d4 = *reinterpret_cast<const float4 *>(bd + ((ch ^ sw) << 4));
                        float4 g4 = *reinterpret_cast<const float4 *>(bg + ((ch ^ sw) << 4));
                        float dd[4] = {d4.x, d4.y, d4.z, d4.w}, gg[4] = {g4.x, g4.y, g4.z, g4.w};
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            int c = 4 * ch + k;
                            float vv = v[half * 16 + c] * cp[c];
                            q = fmaf(dd[k], vv, q);
                            p = fmaf(gg[k], vv, p);
                            sacc = fmaf(cp[kRBN + c], dd[k], sacc);
                            tacc = fmaf(cp[2 * kRBN + c], gg[k], tacc);
                        }
                    }
                    ++consumed;
                    // every epilogue thread is done with buffer e: refill it.
                    // The reads above are generic-proxy and the refill is a TMA
                    // write (async proxy); the barrier alone does not order the
                    // two, and a refill that landed before a slow warp's loads
                    // had read the part gave wrong d values in a few rows of one
                    // tile in about one call in 1500 (M=573, N=20 000)
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("bar.sync 1, 128;" ::: "memory");
                    if (leader) issue_next();
                }
                if (fail_code) break;
            }
            if (fail_code) break;
            if (row < args.R) {
                const long R = args.R;
                float *o = args.qpst + ((long)jimg * nct + ct) * 4 * R;
                o[row] = q;
                o[R + row] = p;
                o[2 * R + row] = sacc;
                o[3 * R + row] = tacc;
            }
        }
        if (fail_code) {
            *abort = 1;
            if (leader)
                for (long k = consumed; k < issued; ++k)
                    mbar_wait(efull0 + 8 * (int)(k % kREpiBufs), (uint32_t)(k / kREpiBufs) & 1,
                              kDefaultBudget);
        }
    }
    if (fail_code && lane == 0) *(volatile int *)args.err = fail_code;
    tc_fence_before();
    __syncthreads();
    if (warp == 5) {
        // every MMA has completed before the TMEM is freed
        mbar_wait(done, 0, kDefaultBudget);
        __syncwarp();
        tc_fence_after();
        tmem_dealloc<512>(tmem);
    }
}

// ------------------------------------------------- persistent stage B
// G = U^T W as split-K partial tiles: work item w = (split, tile), tile a
// 128 x 128 block of the ldG x ldG output, split a range of kbps K blocks.
// One CTA per SM takes items blockIdx.x, blockIdx.x + G, ... (round robin, so
// the SMs work on neighbouring items of the same split at the same time and
// share its U^T and W^T rows in L2).  Same roles as stage A: warps 0-3 write
// the scaled partial tile of item i from one TMEM half while warp 5 runs the
// MMAs of item i+1 into the other; warp 4 keeps the 3-stage operand ring
// full across items.  Bounded waits and the abort flag as in stage A.
constexpr int kQStages = 3;
constexpr uint32_t kQStageBytes = 2 * kABytes + 2 * kBNB * kBK * 2;   // 64 KB
constexpr int kQBars = 2 * kQStages + 5;   // full, empty, tfull[2], tempty[2], done
constexpr size_t kQSmem = 1024 + kQStages * (size_t)kQStageBytes + 2 * kBNB * sizeof(float) +
                          8 * kQBars + 16;
static_assert(kQSmem <= 232448, "stage B shared memory above the per-block limit");

struct StageBArgs {
    int nkb;              // K blocks per split
    int nkb_total;        // K blocks in all
    int Mp;
    int ldG;              // rows of a partial tile (a: modes, ldG = ntile x 128)
    int ntile;            // tiles along a
    int ntile_b;          // tiles along b (the J x Mp rows of W^T, all images)
    int ldGb;             // columns of a partial tile (ntile_b x 128)
    int JMp;              // J x Mp
    long nitems;          // ntile x ntile_b x nsplit
    const float *su, *sw; // row scales of U^T (Mp) and W^T (J x Mp, per image)
    float *gpart;         // [nsplit][ldG][ldGb]
    int *err;
    long long budget;
};

__global__ void __launch_bounds__(192, 1) k_stageB_tc(const __grid_constant__ TmaQuad tm,
                                                       const StageBArgs args) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    float *colv = reinterpret_cast<float *>(smem + kQStages * kQStageBytes);   // [2][kBNB]
    uint64_t *bars = reinterpret_cast<uint64_t *>(colv + 2 * kBNB);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + kQBars);
    volatile int *abort = reinterpret_cast<volatile int *>(tmem_slot + 1);
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * kQStages,
                   tfull0 = empty0 + 8 * kQStages, tempty0 = tfull0 + 16, done = tempty0 + 16;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long budget = args.budget;
    const long G = gridDim.x;
    const long nloc = args.nitems > (long)blockIdx.x ? (args.nitems - 1 - blockIdx.x) / G + 1 : 0;
    const int tiles = args.ntile * args.ntile_b;
    constexpr uint32_t kIdesc = idesc_f16(kBM, kBNB);

    if (threadIdx.x == 0) {
        for (int s = 0; s < kQStages; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int j = 0; j < 2; ++j) {
            mbar_init(tfull0 + 8 * j, 1);
            mbar_init(tempty0 + 8 * j, 128);
        }
        mbar_init(done, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 5) tmem_alloc<512>(smem_u32(tmem_slot));
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // barriers and TMEM are set up; global memory only after the kernels
    // before this one in the stream have completed
    pdl_enter();
    int fail_code = 0;

    if (warp == 4) {
        if (lane == 0) {
            // ---- TMA producer
            long g = 0;
            for (long i = 0; i < nloc && !fail_code; ++i) {
                long w = blockIdx.x + i * G;
                int split = (int)(w / tiles), tile = (int)(w % tiles);
                int arow = (tile / args.ntile_b) * kBM, brow = (tile % args.ntile_b) * kBNB;
                int kb0 = split * args.nkb, nkb = min(args.nkb, args.nkb_total - kb0);
                for (int kb = 0; kb < nkb; ++kb, ++g) {
                    int s = (int)(g % kQStages);
                    uint32_t n = (uint32_t)(g / kQStages);
                    if (g >= kQStages && !mbar_wait_ab(empty0 + 8 * s, (n & 1) ^ 1, budget, abort)) {
                        fail_code = 1;
                        break;
                    }
                    uint32_t base = smem_u32(smem + s * kQStageBytes);
                    uint32_t bar = full0 + 8 * s;
                    int kx = (kb0 + kb) * kBK;
                    mbar_expect_tx(bar, kQStageBytes);
                    tma_load_2d(base, &tm.a_hi, bar, kx, arow);
                    tma_load_2d(base + kABytes, &tm.a_lo, bar, kx, arow);
                    tma_load_2d(base + 2 * kABytes, &tm.b_hi, bar, kx, brow);
                    tma_load_2d(base + 2 * kABytes + kBNB * kBK * 2, &tm.b_lo, bar, kx, brow);
                }
            }
            if (fail_code) {
                *abort = 1;
                for (long gg = g > kQStages ? g - kQStages : 0; gg < g; ++gg)
                    mbar_wait(full0 + 8 * (int)(gg % kQStages), (uint32_t)(gg / kQStages) & 1,
                              kDefaultBudget);
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            // ---- MMA issuer: item i into TMEM half (i & 1)
            long g = 0;
            for (long i = 0; i < nloc && !fail_code; ++i) {
                long w = blockIdx.x + i * G;
                int split = (int)(w / tiles);
                int kb0 = split * args.nkb, nkb = min(args.nkb, args.nkb_total - kb0);
                int j = (int)(i & 1);
                uint32_t u = (uint32_t)(i >> 1);
                if (i >= 2 && !mbar_wait_ab(tempty0 + 8 * j, (u - 1) & 1, budget, abort)) {
                    fail_code = 2;
                    break;
                }
                tc_fence_after();
                const uint32_t d0 = tmem + 256 * j, d1 = d0 + 128;
                for (int kb = 0; kb < nkb; ++kb, ++g) {
                    int s = (int)(g % kQStages);
                    uint32_t n = (uint32_t)(g / kQStages);
                    if (!mbar_wait_ab(full0 + 8 * s, n & 1, budget, abort)) {
                        fail_code = 2;
                        break;
                    }
                    tc_fence_after();
                    uint32_t base = smem_u32(smem + s * kQStageBytes);
#pragma unroll
                    for (int kk = 0; kk < kBK / 16; ++kk) {
                        uint64_t ah = sdesc_sw128(base + kk * 32);
                        uint64_t al = sdesc_sw128(base + kABytes + kk * 32);
                        uint64_t bh = sdesc_sw128(base + 2 * kABytes + kk * 32);
                        uint64_t bl = sdesc_sw128(base + 2 * kABytes + kBNB * kBK * 2 + kk * 32);
                        uint32_t acc = (kb | kk) != 0;
                        mma_f16(d0, ah, bh, kIdesc, acc);
                        mma_f16(d1, ah, bl, kIdesc, acc);
                        mma_f16(d1, al, bh, kIdesc, 1);
                    }
                    mma_commit(empty0 + 8 * s);
                }
                if (fail_code) break;
                mma_commit(tfull0 + 8 * j);
            }
            if (fail_code) *abort = 1;
            mma_commit(done);   // tracks every MMA issued, also after a failure
        }
    } else {
        // ---- epilogue (warps 0-3): thread = tile row = TMEM lane
        const int row_in = warp * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
        for (long i = 0; i < nloc; ++i) {
            long w = blockIdx.x + i * G;
            int split = (int)(w / tiles), tile = (int)(w % tiles);
            int arow = (tile / args.ntile_b) * kBM, brow = (tile % args.ntile_b) * kBNB;
            const int j = (int)(i & 1);
            const uint32_t u = (uint32_t)(i >> 1);
            // W^T row scales of this tile's columns (two buffers: a thread is at
            // most one item ahead of the slowest, see the barrier below)
            float *cv = colv + j * kBNB;
            {
                int c = brow + row_in;
                cv[row_in] = c < args.JMp ? args.sw[c] : 0.f;
            }
            const int a = arow + row_in;
            const float sa = a < args.Mp ? args.su[a] : 0.f;
            bool ok = mbar_wait_ab(tfull0 + 8 * j, u & 1, budget, abort);
            __syncwarp();
            if (epi_sync_or(!ok)) {   // also publishes cv
                fail_code = 3;
                break;
            }
            tc_fence_after();
            float *dst = args.gpart + (long)split * args.ldG * args.ldGb + (long)a * args.ldGb + brow;
#pragma unroll 1
            for (int ch = 0; ch < kBNB / 32; ++ch) {
                float v[32];
                tmem_combined(lane_base + 256 * j, ch * 32, 128, v);
                if (ch == kBNB / 32 - 1) {
                    tc_fence_before();
                    mbar_arrive(tempty0 + 8 * j);
                }
                float4 *d4 = reinterpret_cast<float4 *>(dst + ch * 32);
                const float *cp = cv + ch * 32;
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    d4[q] = make_float4(v[4 * q] * sa * cp[4 * q], v[4 * q + 1] * sa * cp[4 * q + 1],
                                        v[4 * q + 2] * sa * cp[4 * q + 2],
                                        v[4 * q + 3] * sa * cp[4 * q + 3]);
            }
        }
        if (fail_code) *abort = 1;
    }
    if (fail_code && lane == 0) *(volatile int *)args.err = fail_code;
    tc_fence_before();
    __syncthreads();
    if (warp == 5) {
        mbar_wait(done, 0, kDefaultBudget);
        __syncwarp();
        tc_fence_after();
        tmem_dealloc<512>(tmem);
    }
}

// --------------------------------------------------------- data movers
__device__ __forceinline__ void split_f16(float x, __half &hi, __half &lo) {
    hi = __float2half_rn(x);
    lo = __float2half_rn((x - __half2float(hi)) * kLoScale);
}

__device__ __forceinline__ void atomic_max_pos(float *addr, float v) {
    // non-negative floats order like their bit patterns
    atomicMax(reinterpret_cast<int *>(addr), __float_as_int(v));
}

// Column maxima of |D| and |F| (R x M float64) for the per-mode scales.
__global__ void k_colmax(const double *__restrict__ D, const double *__restrict__ F, long R,
                         int M, long rows_per_block, float *__restrict__ dmax,
                         float *__restrict__ fmax) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    long rb = blockIdx.y * rows_per_block, re = min(R, rb + rows_per_block);
    float a = 0.f, b = 0.f;
    for (long r = rb; r < re; ++r) {
        a = fmaxf(a, (float)fabs(D[r * M + m]));
        b = fmaxf(b, (float)fabs(F[r * M + m]));
    }
    atomic_max_pos(dmax + m, a);
    atomic_max_pos(fmax + m, b);
}

// Scales of the operands: sd (mode axis of stage A), su = f_Y sd (rows of
// U^T), fmax (column maxima of F); zero columns get 1, padding gets 1 / 0.
__global__ void k_scales(const float *__restrict__ dmax, const double *__restrict__ fY, int M,
                         int Mp, float *__restrict__ sd, float *__restrict__ su,
                         float *__restrict__ fmx, double *__restrict__ rsd,
                         double *__restrict__ rsu) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= Mp) return;
    if (m < M) {
        float s = dmax[m] > 0.f ? dmax[m] : 1.f;
        sd[m] = s;
        float u = (float)(fY[m] * (double)s);
        su[m] = u > 0.f ? u : 1.f;
        if (!(fmx[m] > 0.f)) fmx[m] = 1.f;
    } else {
        sd[m] = 1.f;
        su[m] = 1.f;
        fmx[m] = 0.f;
    }
    // float64 reciprocals for the operand preparation
    rsd[m] = 1.0 / (double)sd[m];
    rsu[m] = 1.0 / (double)su[m];
}

// Resident operands from the float64 image rows D, F (R x M):
//   d_hi/d_lo  (R x Mp)  limbs of D[r][m] / sd_m   (stage A operand)
//   d32, g32   (R x Mp)  D and f_psi * F in fp32    (stage A epilogue)
// Rows r over blockIdx.y, modes m over the x dimension (no 64-bit division
// per element); the mode scales come as float64 reciprocals (a division per
// element cost most of this pass: float64 runs at 2 FMA per cycle per SM).
__global__ void k_prep_rows(const double *__restrict__ D, const double *__restrict__ F,
                            const double *__restrict__ fpsi, const double *__restrict__ rsd, long R,
                            int M, int Mp, __half *__restrict__ d_hi, __half *__restrict__ d_lo,
                            float *__restrict__ d32, float *__restrict__ g32) {
    for (long r = blockIdx.y; r < R; r += gridDim.y)
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < Mp; m += gridDim.x * blockDim.x) {
        const long e = r * Mp + m;
        float x = 0.f, g = 0.f, xs = 0.f;
        if (m < M) {
            double dv = D[r * M + m];
            x = (float)dv;
            xs = (float)(dv * rsd[m]);
            g = (float)(fpsi[m] * F[r * M + m]);
        }
        __half h, l;
        split_f16(xs, h, l);
        d_hi[e] = h;
        d_lo[e] = l;
        d32[e] = x;
        g32[e] = g;
    }
}

// Transposed operands (Mp x Rp) through 32 x 32 shared tiles:
//   ut_hi/ut_lo  limbs of U[r][a] / su_a   (stage B A operand)
//   ut32, ft32   U and F in fp32            (W build, force average)
__global__ void k_prep_cols(const double *__restrict__ D, const double *__restrict__ F,
                            const double *__restrict__ fY, const double *__restrict__ rsu, long R,
                            int M, long Rp, __half *__restrict__ ut_hi, __half *__restrict__ ut_lo,
                            float *__restrict__ ut32, float *__restrict__ ft32) {
    __shared__ double tu[32][33];
    __shared__ float tf[32][33];
    long r0 = (long)blockIdx.x * 32;
    int m0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        long r = r0 + k;
        int m = m0 + threadIdx.x;
        double u = 0.0;
        float f = 0.f;
        if (r < R && m < M) {
            u = fY[m] * D[r * M + m];
            f = (float)F[r * M + m];
        }
        tu[k][threadIdx.x] = u;
        tf[k][threadIdx.x] = f;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        int m = m0 + k;
        long r = r0 + threadIdx.x;
        if (r < Rp) {
            double u = tu[threadIdx.x][k];
            __half h, l;
            split_f16((float)(u * rsu[m]), h, l);
            long o = (long)m * Rp + r;
            ut_hi[o] = h;
            ut_lo[o] = l;
            ut32[o] = (float)u;
            ft32[o] = tf[threadIdx.x][k];
        }
    }
}

// Per call: Y1 row n scaled by sd (mode axis) and by 1/t_n, t_n its max; one
// block per row.  Also the epilogue vectors f_Y*R1, R1/f_psi, and the reset
// of the alpha / beta maxima.
// Where k_prep_y1 reads Y1 and R1: the context's buffers (written by the
// caller or the psi unpack), or psi itself, unpacked on the fly with the
// unpack's formulas for the plain and transposed layouts
// (Modules/DynamicalLanczos.py:2887-2948, :3009-3053): row n of Y1 from the
// upper-triangle sectors of psi, R1 = psi's R sector.
struct Y1FromBuffers {
    const double *Y1, *R1;
    int M;
    __device__ double y(int n, int m) const { return Y1[(long)n * M + m]; }
    __device__ double r(int n) const { return R1[n]; }
};
struct Y1FromPsi {
    const double *psi;
    const double *cty, *ctra;   // transposed layout's per-pair factors; null: plain
    int M;
    long H;
    int ignore_v3;
    __device__ double y(int n, int m) const {
        const int i = min(n, m), j = max(n, m);
        const long k = (long)i * M - (long)i * (i - 1) / 2 + (j - i);
        const double yv = psi[M + k];
        if (!cty) return yv;
        return yv * cty[k] + psi[M + H + k] * ctra[k];
    }
    __device__ double r(int n) const { return ignore_v3 ? 0.0 : psi[n]; }
};

// The perturbations of one call (one, or the two of a bi-Lanczos step):
// the preparation kernels take perturbation blockIdx.y and write its outputs
// at its image offset
template <class Src>
struct SrcPair {
    Src s[2];
};

template <class Src>
__global__ void k_prep_y1(const SrcPair<Src> sp, const double *__restrict__ fY,
                          const double *__restrict__ fpsi, const float *__restrict__ sd, int M,
                          int Mp, __half *__restrict__ y_hi, __half *__restrict__ y_lo,
                          float *__restrict__ tcol, float *__restrict__ vs,
                          float *__restrict__ vt, float *__restrict__ absmax) {
    pdl_enter();
    __shared__ float red[32];
    const Src &src = sp.s[blockIdx.y];
    y_hi += blockIdx.y * (long)Mp * Mp;
    y_lo += blockIdx.y * (long)Mp * Mp;
    tcol += blockIdx.y * Mp;
    vs += blockIdx.y * Mp;
    vt += blockIdx.y * Mp;
    absmax += 2 * blockIdx.y;
    int n = blockIdx.x;
    float mx = 0.f;
    for (int m = threadIdx.x; m < Mp; m += blockDim.x)
        if (n < M && m < M) mx = fmaxf(mx, fabsf((float)src.y(n, m) * sd[m]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) red[0] = v;
    }
    __syncthreads();
    float t = red[0] > 0.f ? red[0] : 1.f;
    float inv = 1.f / t;
    for (int m = threadIdx.x; m < Mp; m += blockDim.x) {
        float x = (n < M && m < M) ? (float)src.y(n, m) * sd[m] * inv : 0.f;
        __half h, l;
        split_f16(x, h, l);
        y_hi[(long)n * Mp + m] = h;
        y_lo[(long)n * Mp + m] = l;
    }
    if (threadIdx.x == 0) {
        tcol[n] = n < M ? t : 0.f;
        const double r1 = n < M ? src.r(n) : 0.0;
        vs[n] = n < M ? (float)(fY[n] * r1) : 0.f;
        vt[n] = n < M ? (float)(r1 / fpsi[n]) : 0.f;
        if (n == 0) { absmax[0] = 0.f; absmax[1] = 0.f; }
    }
}

// Y1 of one perturbation as double-float pairs (M x M), read from psi or the
// buffers once, so that the image preparation below does not unpack psi for
// every one of its md^2 products per entry
template <class Src>
__global__ void k_y1_df(const SrcPair<Src> sp, int M, float2 *__restrict__ y1) {
    pdl_enter();
    const Src &src = sp.s[blockIdx.y];
    y1 += blockIdx.y * (long)M * M;
    const int n = blockIdx.x;
    for (int m = threadIdx.x; m < M; m += blockDim.x) y1[(long)n * M + m] = split_f64(src.y(n, m));
}

// The same for perturbation-side symmetry images (symmetry.cu): block
// (j, n) forms row n of Y1_j = S_j^T Y1 S_j, and the epilogue vectors of image
// j, (S_j^T (f_Y R1)) and (S_j^T R1) / f_psi, all at j*Mp + n.  The sandwich
// runs in double-float (k_y1_df's Y1 and sc_val2: GB300's float64 rate made
// the md^2 products per entry the kernel's cost); the row is staged in dynamic
// shared memory (Mp floats) between its max and its limbs.
template <class Src>
__global__ void k_prep_y1_img(const SrcPair<Src> sp, const float2 *__restrict__ y1,
                              const int *__restrict__ sc_idx,
                              const double *__restrict__ sc_val,
                              const float2 *__restrict__ sc_val2, int md,
                              const double *__restrict__ fY, const double *__restrict__ fpsi,
                              const float *__restrict__ sd, int M, int Mp,
                              __half *__restrict__ y_hi, __half *__restrict__ y_lo,
                              float *__restrict__ tcol, float *__restrict__ vs,
                              float *__restrict__ vt, float *__restrict__ absmax) {
    pdl_enter();
    extern __shared__ float yrow[];
    __shared__ float red[32];
    // perturbation blockIdx.y: its J images at image offset blockIdx.y * J
    const Src &src = sp.s[blockIdx.y];
    const long J = gridDim.x / Mp, io = blockIdx.y * J;
    y1 += blockIdx.y * (long)M * M;
    y_hi += io * Mp * Mp;
    y_lo += io * Mp * Mp;
    tcol += io * Mp;
    vs += io * Mp;
    vt += io * Mp;
    absmax += 2 * io;
    const int n = blockIdx.x % Mp, j = blockIdx.x / Mp;
    const int *ia = sc_idx + ((long)j * M + (n < M ? n : 0)) * md;
    const double *va = sc_val + ((long)j * M + (n < M ? n : 0)) * md;
    const float2 *va2 = sc_val2 + ((long)j * M + (n < M ? n : 0)) * md;
    float mx = 0.f;
    for (int m = threadIdx.x; m < Mp; m += blockDim.x) {
        float ys = 0.f;
        if (n < M && m < M) {
            const int *ib = sc_idx + ((long)j * M + m) * md;
            const float2 *vb2 = sc_val2 + ((long)j * M + m) * md;
            float s = 0.f, c = 0.f;
            for (int p = 0; p < md && ia[p] >= 0; ++p) {
                float is = 0.f, ic = 0.f;
                const float2 *row = y1 + (long)ia[p] * M;
                for (int q = 0; q < md && ib[q] >= 0; ++q) df_fma_acc(is, ic, vb2[q], row[ib[q]]);
                df_fma_acc(s, c, va2[p], df_norm(is, ic));
            }
            ys = (s + c) * sd[m];
        }
        yrow[m] = ys;
        mx = fmaxf(mx, fabsf(ys));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) red[0] = v;
    }
    __syncthreads();
    const float t = red[0] > 0.f ? red[0] : 1.f, inv = 1.f / t;
    const long row = (long)j * Mp + n;
    for (int m = threadIdx.x; m < Mp; m += blockDim.x) {
        __half h, l;
        split_f16(yrow[m] * inv, h, l);
        y_hi[row * Mp + m] = h;
        y_lo[row * Mp + m] = l;
    }
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        if (n < M)
            for (int p = 0; p < md && ia[p] >= 0; ++p) {
                const double r1 = src.r(ia[p]);
                a = fma(va[p], fY[ia[p]] * r1, a);
                b = fma(va[p], r1, b);
            }
        tcol[row] = n < M ? t : 0.f;
        vs[row] = n < M ? (float)a : 0.f;
        vt[row] = n < M ? (float)(b / fpsi[n]) : 0.f;
        if (n == 0) { absmax[2 * j] = 0.f; absmax[2 * j + 1] = 0.f; }   // per image
    }
}

// Row scalars from the stage A partials (sums in double-float), and max |alpha|,
// max |beta| of each perturbation image for its W scales.  Block
// (x, image j) takes rows r = j*Nr + i of configuration rows i (J = 1: the
// image rows themselves, i = r).
__global__ void k_rows_mixed(const float *__restrict__ qpst, int nct, long Nr, int rho_div,
                             const double *__restrict__ rho, int apply_d4,
                             float4 *__restrict__ abcc, float *__restrict__ absmax) {
    pdl_enter();
    const long jj = blockIdx.y;
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const long r = jj * Nr + i;
    absmax += 2 * jj;
    float ma = 0.f, mb = 0.f;
    if (i < Nr) {
        // the column-tile sums and the combinations in double-float: the
        // results are rounded to fp32, and float64 here made the kernel
        // float64-pipe bound at 96 images (0.96 M rows)
        const float *base = qpst + jj * nct * 4 * Nr;
        float qs = 0.f, qc = 0.f, ps = 0.f, pc = 0.f, ss = 0.f, sc = 0.f, ts = 0.f, tc = 0.f;
        for (int ct = 0; ct < nct; ++ct) {
            const float *o = base + (long)ct * 4 * Nr;
            df_two_sum_acc(qs, qc, o[i]);
            df_two_sum_acc(ps, pc, o[Nr + i]);
            df_two_sum_acc(ss, sc, o[2 * Nr + i]);
            df_two_sum_acc(ts, tc, o[3 * Nr + i]);
        }
        const float2 q = df_norm(qs, qc), p = df_norm(ps, pc), s3 = df_norm(ss, sc),
                     t3 = df_norm(ts, tc);
        const float2 rw = split_f64(rho[i / rho_div]);
        // 1/3 and 1/6 as double-float constants
        const float2 third = make_float2(0.333333343f, -9.93410776e-09f);
        const float2 sixth = make_float2(0.166666672f, -4.96705388e-09f);
        const float d4 = apply_d4 ? 1.f : 0.f;
        const float2 a = df_add(df_mul(s3, third), make_float2(-d4 * 0.125f * q.x, -d4 * 0.125f * q.y));
        const float2 b = df_add(df_mul(t3, third), make_float2(-d4 * 0.25f * p.x, -d4 * 0.25f * p.y));
        const float2 c1 = df_mul(q, sixth), c2 = df_mul(p, third);
        const float2 ra = df_mul(rw, a), rb = df_mul(rw, b), r1 = df_mul(rw, c1), r2 = df_mul(rw, c2);
        float4 v = make_float4(ra.x + ra.y, rb.x + rb.y, -(r1.x + r1.y), -(r2.x + r2.y));
        abcc[r] = v;
        ma = fabsf(v.x);
        mb = fabsf(v.y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, o));
        mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, o));
    }
    // one atomic per block and value (same-address atomics serialise)
    __shared__ float red[2][32];
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = ma;
        red[1][threadIdx.x >> 5] = mb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            ma = fmaxf(ma, red[0][k]);
            mb = fmaxf(mb, red[1][k]);
        }
        atomic_max_pos(absmax, ma);
        atomic_max_pos(absmax + 1, mb);
    }
}

// W^T[b][r] = (alpha_r F^T[b][r] + beta_r/2 U^T[b][r]) / sw_b as fp16 limbs,
// sw_b = max|alpha| fmax_b + max|beta|/2 su_b (maxima of the image); and the
// force-average partials fpart[chunk][b] = sum_r c1_r F^T[b][r] + c2_r U^T[b][r].
// Contexts without symmetry images: block (b group, r chunk) reads its F^T
// and U^T tile once and writes the W^T tiles of the nimg <= 2 perturbations
// of the call (the L and L^T applications of a bi-Lanczos step): image j's row
// scalars at j*R, its maxima at 2j, its W^T rows and scales at j*Mp, its force
// partials at j*nchunk*M.  89.5 us against 120 per step at M=573, N=50 000.
// (With 96 symmetry images in one block per tile: 261 us against 188 for
// k_wbuild_img, and 277 us with one image per block in this form.)
constexpr int kWRows = 8;      // b rows per block
constexpr int kWChunk = 1024;  // r per block (256 threads x 4 r)
constexpr int kWPair = 2;      // images per block
__global__ void __launch_bounds__(256, 2) k_wbuild_pair(const float *__restrict__ ft32,
                                                const float *__restrict__ ut32,
                                                const float4 *__restrict__ abcc,
                                                const float *__restrict__ absmax,
                                                const float *__restrict__ fmax,
                                                const float *__restrict__ su, long R, long Rp,
                                                int M, int Mp, int nimg,
                                                __half *__restrict__ wt_hi,
                                                __half *__restrict__ wt_lo,
                                                float *__restrict__ sw_out,
                                                float *__restrict__ fpart) {
    pdl_enter();
    __shared__ float red[kWRows][8];
    const int b0 = blockIdx.x * kWRows;
    // Rp is a multiple of 64 and r of 4, so each 4-group is in bounds of the
    // padded rows; rows r >= R carry alpha = beta = c1 = c2 = 0 there
    const long r = (long)blockIdx.y * kWChunk + 4 * threadIdx.x;
    const bool rin = r < Rp;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float4 f4[kWRows], u4[kWRows];
#pragma unroll
    for (int k = 0; k < kWRows; ++k) {
        const long o = (long)(b0 + k) * Rp + r;
        const bool in = rin && b0 + k < M;
        f4[k] = in ? *reinterpret_cast<const float4 *>(ft32 + o) : make_float4(0.f, 0.f, 0.f, 0.f);
        u4[k] = in ? *reinterpret_cast<const float4 *>(ut32 + o) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int j = 0; j < kWPair; ++j) {
        if (j >= nimg) break;   // uniform over the block
        const float amax = absmax[2 * j], bmax = absmax[2 * j + 1];
        float4 w4[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            w4[q] = (rin && r + q < R) ? abcc[(long)j * R + r + q] : make_float4(0.f, 0.f, 0.f, 0.f);
        __half *wh = wt_hi + (long)j * Mp * Rp, *wl = wt_lo + (long)j * Mp * Rp;
        float facc[kWRows];
#pragma unroll
        for (int k = 0; k < kWRows; ++k) {
            const int b = b0 + k;
            facc[k] = 0.f;
            if (b >= M) continue;
            float sw = amax * fmax[b] + 0.5f * bmax * su[b];
            if (!(sw > 0.f)) sw = 1.f;
            const float inv = 1.f / sw;
            if (blockIdx.y == 0 && threadIdx.x == 0) sw_out[(long)j * Mp + b] = sw;
            if (!rin) continue;
            const float ff[4] = {f4[k].x, f4[k].y, f4[k].z, f4[k].w};
            const float uu[4] = {u4[k].x, u4[k].y, u4[k].z, u4[k].w};
            __align__(8) __half hh[4], ll[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float x = (w4[q].x * ff[q] + 0.5f * w4[q].y * uu[q]) * inv;
                split_f16(x, hh[q], ll[q]);
                facc[k] = fmaf(w4[q].z, ff[q], fmaf(w4[q].w, uu[q], facc[k]));
            }
            const long o = (long)b * Rp + r;
            *reinterpret_cast<uint2 *>(wh + o) = *reinterpret_cast<const uint2 *>(hh);
            *reinterpret_cast<uint2 *>(wl + o) = *reinterpret_cast<const uint2 *>(ll);
        }
#pragma unroll
        for (int k = 0; k < kWRows; ++k) {
            float v = facc[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) red[k][wid] = v;
        }
        __syncthreads();
        if (threadIdx.x < kWRows) {
            const int b = b0 + threadIdx.x;
            float sacc = 0.f;
            for (int w8 = 0; w8 < 8; ++w8) sacc += red[threadIdx.x][w8];
            if (b < M) fpart[((long)j * gridDim.y + blockIdx.y) * M + b] = sacc;
        }
        __syncthreads();   // red is reused by the next image
    }
}

// Contexts with symmetry images: the same W^T limbs and force partials with
// one image per block, block (b group, r chunk, image j) (the fp32 F^T and U^T
// tiles sit in L2 there and the grid needs the image dimension): row scalars
// of image j at j*R, its maxima at 2j, W^T rows and scales at j*Mp, force
// partials at j*nchunk*M.
constexpr int kWChunkImg = 2048;  // r per block (256 threads x 4 r x 2 passes)
__global__ void __launch_bounds__(256) k_wbuild_img(const float *__restrict__ ft32,
                                                const float *__restrict__ ut32,
                                                const float4 *__restrict__ abcc,
                                                const float *__restrict__ absmax,
                                                const float *__restrict__ fmax,
                                                const float *__restrict__ su, long R, long Rp,
                                                int M, int Mp, __half *__restrict__ wt_hi,
                                                __half *__restrict__ wt_lo,
                                                float *__restrict__ sw_out,
                                                float *__restrict__ fpart) {
    pdl_enter();
    abcc += blockIdx.z * R;
    wt_hi += (long)blockIdx.z * Mp * Rp;
    wt_lo += (long)blockIdx.z * Mp * Rp;
    fpart += (long)blockIdx.z * gridDim.y * M;
    absmax += 2 * blockIdx.z;
    sw_out += (long)blockIdx.z * Mp;
    __shared__ float red[kWRows][8];
    int b0 = blockIdx.x * kWRows;
    long r0 = (long)blockIdx.y * kWChunkImg;
    const float amax = absmax[0], bmax = absmax[1];
    float inv[kWRows], facc[kWRows];
#pragma unroll
    for (int k = 0; k < kWRows; ++k) {
        int b = b0 + k;
        float sw = b < M ? amax * fmax[b] + 0.5f * bmax * su[b] : 1.f;
        if (!(sw > 0.f)) sw = 1.f;
        inv[k] = 1.f / sw;
        facc[k] = 0.f;
        if (blockIdx.y == 0 && threadIdx.x == 0 && b < M) sw_out[b] = sw;
    }
    // Rp is a multiple of 64 and r0 of 2048, so each 4-group is in bounds of
    // the padded rows; rows r >= R carry alpha = beta = c1 = c2 = 0 there.
#pragma unroll
    for (int pass = 0; pass < kWChunkImg / 1024; ++pass) {
        long r = r0 + pass * 1024 + 4 * threadIdx.x;
        if (r >= Rp) break;
        float4 w4[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            w4[q] = (r + q < R) ? abcc[r + q] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < kWRows; ++k) {
            int b = b0 + k;
            if (b >= M) break;
            long o = (long)b * Rp + r;
            float4 f4 = *reinterpret_cast<const float4 *>(ft32 + o);
            float4 u4 = *reinterpret_cast<const float4 *>(ut32 + o);
            float ff[4] = {f4.x, f4.y, f4.z, f4.w}, uu[4] = {u4.x, u4.y, u4.z, u4.w};
            __align__(8) __half hh[4], ll[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float x = (w4[q].x * ff[q] + 0.5f * w4[q].y * uu[q]) * inv[k];
                split_f16(x, hh[q], ll[q]);
                facc[k] = fmaf(w4[q].z, ff[q], fmaf(w4[q].w, uu[q], facc[k]));
            }
            *reinterpret_cast<uint2 *>(wt_hi + o) = *reinterpret_cast<const uint2 *>(hh);
            *reinterpret_cast<uint2 *>(wt_lo + o) = *reinterpret_cast<const uint2 *>(ll);
        }
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kWRows; ++k) {
        float v = facc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[k][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < kWRows) {
        int b = b0 + threadIdx.x;
        float s = 0.f;
        for (int w8 = 0; w8 < 8; ++w8) s += red[threadIdx.x][w8];
        if (b < M) fpart[(long)blockIdx.y * M + b] = s;
    }
}

// Split-K sum and finalisation in one pass: one block per 8-row slab of a
// 32 x 32 tile pair (A, B), A <= B.  G over the partial tiles is formed for the
// slab's transposed part of tile (B, A) first (kept in shared memory) and then
// for its part of (A, B), each element as a
// compensated fp32 sum over the splits in split order, and
// d2v[a][b] = d2v[b][a] = -(G[a][b] + G[b][a]) / norm is written without a
// float64 G round trip.  Blocks with A = 0 also finish f for the columns of
// tile B.  G_s[a][b] = gpart[s * stride + a * lda + b] (one image's columns of
// the partial tiles).
__device__ __forceinline__ double gsum_one(const float *__restrict__ g, int nsplit, long stride) {
    float sum = 0.f, comp = 0.f;
    int s = 0;
    // eight loads in flight per thread (the sum is latency-bound)
    for (; s + 8 <= nsplit; s += 8) {
        float v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = g[(long)(s + u) * stride];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            float y = v[u] - comp;
            float t = sum + y;
            comp = (t - sum) - y;
            sum = t;
        }
    }
    for (; s < nsplit; ++s) {
        float y = g[(long)s * stride] - comp;
        float t = sum + y;
        comp = (t - sum) - y;
        sum = t;
    }
    return (double)sum - (double)comp;
}

__global__ void __launch_bounds__(256) k_gfinal(const float *__restrict__ gpart, int nsplit,
                                                long lda, long stride, int M, int Mp,
                                                const float *__restrict__ fpart, int nfchunk,
                                                double norm, double *__restrict__ f,
                                                double *__restrict__ d2v, double *__restrict__ f2,
                                                double *__restrict__ d2v2) {
    pdl_enter();
    // perturbation blockIdx.y of the call: its G columns and force partials,
    // its outputs
    if (blockIdx.y) {
        gpart += Mp;
        fpart += (long)nfchunk * M;
        f = f2;
        d2v = d2v2;
    }
    __shared__ double tr[32][9];    // G over rows b of tile B, the slab's 8 columns a: [b][a]
    __shared__ double red[8][33];
    // (pair, slab): pair index -> (A, B), A <= B, row-major over the upper
    // triangle of tiles; slab = 8 rows a of tile A
    const int nt = (M + 31) / 32;
    const int slab = blockIdx.x & 3;
    int A = 0, rem = blockIdx.x >> 2;
    while (rem >= nt - A) {
        rem -= nt - A;
        ++A;
    }
    const int B = A + rem;
    const double inv = 1.0 / norm;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 8 x 32
    const int a0 = A * 32 + slab * 8, b0 = B * 32;
    {
        // G[b][a] for the 32 rows b of tile B and the slab's 8 columns a; lanes
        // along a, so that a warp reads 4 rows x 8 consecutive floats (4 sectors)
        int ao = threadIdx.x & 7, bo = threadIdx.x >> 3;
        int b = b0 + bo, a = a0 + ao;
        tr[bo][ao] = (a < M && b < M) ? gsum_one(gpart + (long)b * lda + a, nsplit, stride) : 0.0;
    }
    __syncthreads();
    {
        int a = a0 + ty, b = b0 + tx;                         // G[a][b], coalesced in b
        if (a < M && b < M) {
            double v = -(gsum_one(gpart + (long)a * lda + b, nsplit, stride) + tr[tx][ty]) * inv;
            d2v[(long)a * M + b] = v;
            if (A != B) d2v[(long)b * M + a] = v;
        }
    }
    if (A == 0 && slab == 0) {
        // f for the block's 32 columns of tile B: 8 chunk-strided partials per column
        int e = b0 + tx;
        double acc = 0;
        if (e < M)
            for (int ch = ty; ch < nfchunk; ch += 8) acc += (double)fpart[(long)ch * M + e];
        red[ty][tx] = acc;
        __syncthreads();
        if (ty == 0 && e < M) {
            double sum = 0;
            for (int k = 0; k < 8; ++k) sum += red[k][tx];
            f[e] = sum * inv;
        }
    }
}

// ------------------------------------------------------------- host side
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2D fp16 tensor (inner x outer, row pitch inner*2 bytes), box 64 x box_rows,
// 128-byte swizzle, zero fill out of bounds.
static int make_map(CUtensorMap *m, const void *base, uint64_t inner, uint64_t outer,
                    uint32_t box_rows) {
    auto fn = encode_fn();
    if (!fn) { set_error("cuTensorMapEncodeTiled unavailable"); return TDSCHA_ERR_CUDA; }
    if ((reinterpret_cast<uintptr_t>(base) & 15) || ((inner * 2) & 15) || inner % kBK ||
        box_rows == 0 || box_rows > 256) {
        set_error("tensor map: misaligned base or pitch, or bad box");
        return TDSCHA_ERR_ARG;
    }
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBK, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base), dims, strides,
                    box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return TDSCHA_ERR_CUDA; }
    return TDSCHA_OK;
}

// 2D fp32 tensor (inner x outer), box 16 x 128, 64-byte swizzle.
static int make_map_f32(CUtensorMap *m, const void *base, uint64_t inner, uint64_t outer) {
    auto fn = encode_fn();
    if (!fn) { set_error("cuTensorMapEncodeTiled unavailable"); return TDSCHA_ERR_CUDA; }
    if ((reinterpret_cast<uintptr_t>(base) & 15) || ((inner * 4) & 15) || inner % 32) {
        set_error("tensor map (fp32): misaligned base or pitch");
        return TDSCHA_ERR_ARG;
    }
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * 4};
    cuuint32_t box[2] = {(cuuint32_t)kPEpiCols, (cuuint32_t)kBM};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(base), dims, strides,
                    box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled (fp32) failed (%d)", (int)r); return TDSCHA_ERR_CUDA; }
    return TDSCHA_OK;
}


struct MixedExtra {
    TmaQuad tmA, tmB;
    TmaQuad tmA1;             // stage A operand maps for the 192-row B boxes (one accumulator)
    TmaEpi te;
    int bnA = 0;
    float *sd = nullptr, *fmx = nullptr, *su = nullptr, *sw = nullptr, *tcol = nullptr;
    float *vs = nullptr, *vt = nullptr, *absmax = nullptr;
    float *d32 = nullptr;
    float4 *abcc = nullptr;
    float2 *y1df = nullptr;   // symmetry images: Y1 of each perturbation (2 x M x M)
    float *fpart = nullptr;
    int nfchunk = 0;
    int ldG = 0, ntB = 0, nkbB = 0, kbps = 0;
    int ntBb = 0, ldGb = 0;   // stage B tiles / columns along the J x Mp rows of W^T
    int jmax = 1;             // images the per-call buffers hold: 2 J (two perturbations)
    int one_acc = 0;          // stage A with one accumulator per 128 x 192 tile
    double tuned_ms = 0;      // autotuner: time of one application with the chosen shape
    int force_acc = -1;       // TDSCHA_STAGEA_ACC: the stage A kernel fixed by the environment
    std::vector<int> split_cands;
    int nsm = 1;
    long long budget = kDefaultBudget;
};

static MixedExtra *extra(tdscha_ctx *c) { return reinterpret_cast<MixedExtra *>(c->mx.tmaps); }

static void set_stage_a(MixedExtra *x, MixedStore &mx, int one_acc) {
    x->one_acc = one_acc;
    const int bn = one_acc ? kRBN : kPBN;
    x->bnA = std::min(bn, mx.Mp);
    mx.nctile = ceil_div(mx.Mp, bn);
}

static void set_splits(MixedExtra *x, MixedStore &mx, int n) {
    x->kbps = ceil_div(x->nkbB, n);
    mx.nsplit = ceil_div(x->nkbB, x->kbps);
}

// Autotuner of the tensor-core shapes.  For each new (modes, rows, images)
// shape it times one mixed application (stage A kernel: two accumulators on
// 128-wide tiles or one accumulator on 192-wide tiles; stage B split counts
// within the accuracy budget, see split_cands) on the context's own operands,
// one warm-up and three timed calls each, and keeps the fastest; the choice
// is cached per shape for the life of the process, so contexts of one shape
// give the same bits.  TDSCHA_AUTOTUNE=0 keeps the rule-based shape.
static std::mutex g_tune_mu;
struct Tuned {
    int one_acc, nsplit;
    double ms;
};
static std::map<std::array<long, 3>, Tuned> g_tuned;

static int autotune(tdscha_ctx *c) {
    MixedExtra *x = extra(c);
    MixedStore &mx = c->mx;
    if (const char *e = getenv("TDSCHA_AUTOTUNE"))
        if (atoi(e) == 0) return TDSCHA_OK;
    const std::array<long, 3> key{(long)c->M, c->Nrows, (long)c->J};
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
        if (x->force_acc < 0) set_stage_a(x, mx, it->second.one_acc);
        set_splits(x, mx, it->second.nsplit);
        x->tuned_ms = it->second.ms;
        return TDSCHA_OK;
    }
    const int M = c->M;
    // a fixed perturbation of typical magnitude in the per-call buffers
    std::vector<double> r1(M), y1((size_t)M * M);
    for (int a = 0; a < M; ++a) {
        r1[a] = 1.0 / std::sqrt((double)M) * ((a % 3) - 1.0);
        for (int b = 0; b < M; ++b)
            y1[(size_t)a * M + b] = 1e-3 * std::cos(0.37 * (a + 1) * (b + 1));
    }
    TDS_CUDA(cudaMemcpy(c->R1, r1.data(), sizeof(double) * M, cudaMemcpyHostToDevice));
    TDS_CUDA(cudaMemcpy(c->Y1, y1.data(), sizeof(double) * M * M, cudaMemcpyHostToDevice));
    std::vector<int> accs;
    if (x->force_acc >= 0) accs.push_back(x->force_acc);
    else accs = {0, 1};
    cudaEvent_t e0, e1;
    TDS_CUDA(cudaEventCreate(&e0));
    TDS_CUDA(cudaEventCreate(&e1));
    // the candidates run with the default wait budget whatever the context's own
    const long long budget = x->budget;
    x->budget = kDefaultBudget;
    double best = 1e300;
    int best_acc = x->one_acc, best_n = mx.nsplit;
    int rc = TDSCHA_OK;
    for (int acc : accs) {
        for (int n : x->split_cands) {
            set_stage_a(x, mx, acc);
            set_splits(x, mx, n);
            rc = perturb_mixed(c, 1, 0);
            if (rc == TDSCHA_OK && cudaEventRecord(e0, 0) != cudaSuccess) rc = TDSCHA_ERR_CUDA;
            for (int k = 0; k < 3 && rc == TDSCHA_OK; ++k) rc = perturb_mixed(c, 1, 0);
            float ms = 0;
            if (rc == TDSCHA_OK && (cudaEventRecord(e1, 0) != cudaSuccess ||
                                    cudaEventSynchronize(e1) != cudaSuccess ||
                                    cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
                rc = TDSCHA_ERR_CUDA;
            if (rc == TDSCHA_OK) rc = mixed_check_error(c);
            if (rc != TDSCHA_OK) break;
            // a candidate replaces the current best only if more than 1 % faster
            if (ms / 3.0 < best * 0.99) {
                best = ms / 3.0;
                best_acc = acc;
                best_n = n;
            }
        }
        if (rc != TDSCHA_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    x->budget = budget;
    if (rc != TDSCHA_OK) return rc;
    set_stage_a(x, mx, best_acc);
    set_splits(x, mx, best_n);
    x->tuned_ms = best;
    g_tuned[key] = Tuned{best_acc, best_n, best};
    return TDSCHA_OK;
}

int mixed_prepare(tdscha_ctx *c) {
    MixedStore &mx = c->mx;
    const int M = c->M, J = c->J;
    const long R = c->Nrows;   // rows of D, F: image rows, or the N configurations
    mx.Mp = ((M + 63) / 64) * 64;
    mx.Rp = ((R + 63) / 64) * 64;
    const int Mp = mx.Mp;
    const long Rp = mx.Rp;
    MixedExtra *x = new MixedExtra();
    mx.tmaps = x;
    if (const char *b = getenv("TDSCHA_WAIT_BUDGET_CYCLES")) x->budget = atoll(b);
    int force_acc = -1;
    if (const char *e = getenv("TDSCHA_STAGEA_ACC")) force_acc = atoi(e) == 1 ? 1 : 0;
    x->force_acc = force_acc;
    x->one_acc = force_acc == 1;
    const int bnA = x->one_acc ? kRBN : kPBN;
    x->bnA = std::min(bnA, Mp);
    mx.nctile = ceil_div(Mp, bnA);
    const int nct_max = ceil_div(Mp, kPBN);
    {
        int dev = 0, nsm = 0;
        TDS_CUDA(cudaGetDevice(&dev));
        TDS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        x->nsm = std::max(1, nsm);
    }
    x->ldG = ((Mp + kBM - 1) / kBM) * kBM;
    x->ntB = x->ldG / kBM;
    x->ntBb = ceil_div((long)J * Mp, kBNB);
    x->ldGb = x->ntBb * kBNB;
    x->nkbB = (int)(Rp / kBK);
    long split_rows = kSplitRows;
    if (const char *e = getenv("TDSCHA_SPLIT_ROWS")) split_rows = std::max(64L, atol(e));
    int want = std::max(1, ceil_div(R, split_rows));
    want = std::min(want, x->nkbB);
    {
        // among split counts up to `want`, take the one whose grid fills the
        // 152 SMs in whole waves best (ties: more splits)
        const int tiles = x->ntB * x->ntBb;
        int best = want;
        double best_fill = 0;
        for (int n = std::max(1, want / 2); n <= want; ++n) {
            long ctas = (long)tiles * n;
            double fill = (double)ctas / (double)(ceil_div(ctas, 152) * 152L);
            if (fill > best_fill + 1e-9 || (fill > best_fill - 1e-9 && n > best)) {
                best_fill = fill;
                best = n;
            }
        }
        want = best;
    }
    x->kbps = ceil_div(x->nkbB, want);
    mx.nsplit = ceil_div(x->nkbB, x->kbps);
    // split counts the autotuner may pick: accumulations of at most ~1.1 x the
    // split length (the accuracy budget), the best wave fills of 152 SMs
    std::vector<int> split_cands{mx.nsplit};
    {
        const int tiles = x->ntB * x->ntBb;
        const int lo = std::max(1, (int)std::ceil(0.9 * (double)ceil_div(R, split_rows)));
        const int hi = std::min(x->nkbB, 2 * std::max(1, ceil_div(R, split_rows)));
        std::vector<std::pair<double, int>> fills;
        for (int n = lo; n <= hi; ++n) {
            int kb = ceil_div(x->nkbB, n), ns = ceil_div(x->nkbB, kb);
            if (ns != n) continue;
            long ctas = (long)tiles * n;
            fills.push_back({(double)ctas / (double)(ceil_div(ctas, 152) * 152L) + 1e-6 * n, n});
        }
        std::sort(fills.rbegin(), fills.rend());
        for (size_t k = 0; k < fills.size() && split_cands.size() < 4; ++k)
            if (std::find(split_cands.begin(), split_cands.end(), fills[k].second) ==
                split_cands.end())
                split_cands.push_back(fills[k].second);
    }
    x->split_cands = split_cands;
    const int nsplit_max = *std::max_element(split_cands.begin(), split_cands.end());
    // force partial chunks: the r range of one W-build block (per-image form
    // with symmetry images, two-perturbation form without)
    x->nfchunk = ceil_div(R, J > 1 ? kWChunkImg : kWChunk);
    // the per-call buffers hold the images of two perturbations (the L and
    // L^T applications of a bi-Lanczos step in one call)
    const int Jm = 2 * J;
    x->jmax = Jm;
    const int ldGb_max = ceil_div((long)Jm * Mp, kBNB) * kBNB;
    size_t rowN = (size_t)R * Mp, colN = (size_t)Mp * Rp;
    TDS_CUDA(cached_malloc(&mx.d_hi, 2 * rowN));
    TDS_CUDA(cached_malloc(&mx.d_lo, 2 * rowN));
    TDS_CUDA(cached_malloc(&x->d32, 4 * rowN));
    TDS_CUDA(cached_malloc(&mx.g32, 4 * rowN));
    TDS_CUDA(cached_malloc(&mx.ut_hi, 2 * colN));
    TDS_CUDA(cached_malloc(&mx.ut_lo, 2 * colN));
    TDS_CUDA(cached_malloc(&mx.ut32, 4 * colN));
    TDS_CUDA(cached_malloc(&mx.ft32, 4 * colN));
    TDS_CUDA(cached_malloc(&mx.wt_hi, 2 * (size_t)Jm * colN));
    TDS_CUDA(cached_malloc(&mx.wt_lo, 2 * (size_t)Jm * colN));
    TDS_CUDA(cached_malloc(&mx.y1_hi, 2 * (size_t)Jm * Mp * Mp));
    TDS_CUDA(cached_malloc(&mx.y1_lo, 2 * (size_t)Jm * Mp * Mp));
    TDS_CUDA(cached_malloc(&mx.qp, sizeof(float) * 4 * nct_max * (size_t)Jm * R));
    TDS_CUDA(cached_malloc(&mx.gpart, sizeof(float) * (size_t)nsplit_max * x->ldG * ldGb_max));
    float **vecs[] = {&x->sd, &x->fmx, &x->su};
    for (float **v : vecs) TDS_CUDA(cached_malloc(v, sizeof(float) * Mp));
    float **jvecs[] = {&x->tcol, &x->vs, &x->vt, &x->sw};
    for (float **v : jvecs) TDS_CUDA(cached_malloc(v, sizeof(float) * (size_t)Jm * Mp));
    TDS_CUDA(cached_malloc(&x->absmax, sizeof(float) * 2 * Jm));
    TDS_CUDA(cached_malloc(&x->abcc, sizeof(float4) * (size_t)Jm * R));
    TDS_CUDA(cached_malloc(&x->fpart, sizeof(float) * (size_t)Jm * x->nfchunk * M));
    if (J > 1) TDS_CUDA(cached_malloc(&x->y1df, sizeof(float2) * 2 * (size_t)M * M));
    TDS_CUDA(cached_malloc(&c->f2, sizeof(double) * M));
    TDS_CUDA(cached_malloc(&c->d2v2, sizeof(double) * (size_t)M * M));
    TDS_CUDA(cudaHostAlloc(&mx.err_flag, sizeof(int), cudaHostAllocMapped));
    *mx.err_flag = 0;
    TDS_CUDA(cudaMemset(mx.wt_hi, 0, 2 * (size_t)Jm * colN));
    TDS_CUDA(cudaMemset(mx.wt_lo, 0, 2 * (size_t)Jm * colN));
    TDS_CUDA(cudaMemset(x->sw, 0, sizeof(float) * (size_t)Jm * Mp));
    {
        float *dmax = nullptr;
        double *rsc = nullptr;   // 1 / sd and 1 / su in float64 (Mp each)
        TDS_CUDA(cached_malloc(&dmax, sizeof(float) * Mp));
        TDS_CUDA(cached_malloc(&rsc, sizeof(double) * 2 * Mp));
        TDS_CUDA(cudaMemset(dmax, 0, sizeof(float) * Mp));
        TDS_CUDA(cudaMemset(x->fmx, 0, sizeof(float) * Mp));
        long rpb = 512;
        dim3 g(ceil_div(M, 128), ceil_div(R, rpb));
        k_colmax<<<g, 128>>>(c->D, c->F, R, M, rpb, dmax, x->fmx);
        TDS_CHECK_LAUNCH();
        k_scales<<<ceil_div(Mp, 128), 128>>>(dmax, c->fY, M, Mp, x->sd, x->su, x->fmx, rsc,
                                             rsc + Mp);
        TDS_CHECK_LAUNCH();
        TDS_CUDA(cudaDeviceSynchronize());
        cached_free(dmax);
        dim3 gr(ceil_div(Mp, 128), (unsigned)std::min<long>(R, 4096));
        k_prep_rows<<<gr, 128>>>(c->D, c->F, c->fpsi, rsc, R, M, Mp, mx.d_hi, mx.d_lo, x->d32,
                                 mx.g32);
        TDS_CHECK_LAUNCH();
        dim3 gc(ceil_div(Rp, 32), Mp / 32);
        k_prep_cols<<<gc, dim3(32, 8)>>>(c->D, c->F, c->fY, rsc + Mp, R, M, Rp, mx.ut_hi,
                                         mx.ut_lo, mx.ut32, mx.ft32);
        TDS_CHECK_LAUNCH();
        TDS_CUDA(cudaDeviceSynchronize());
        cached_free(rsc);
    }
    TDS_TRY(make_map(&x->tmA.a_hi, mx.d_hi, Mp, R, kBM));
    TDS_TRY(make_map(&x->tmA.a_lo, mx.d_lo, Mp, R, kBM));
    TDS_TRY(make_map(&x->tmA.b_hi, mx.y1_hi, Mp, (uint64_t)Jm * Mp, std::min(kPBN, Mp)));
    TDS_TRY(make_map(&x->tmA.b_lo, mx.y1_lo, Mp, (uint64_t)Jm * Mp, std::min(kPBN, Mp)));
    x->tmA1 = x->tmA;
    TDS_TRY(make_map(&x->tmA1.b_hi, mx.y1_hi, Mp, (uint64_t)Jm * Mp, std::min(kRBN, Mp)));
    TDS_TRY(make_map(&x->tmA1.b_lo, mx.y1_lo, Mp, (uint64_t)Jm * Mp, std::min(kRBN, Mp)));
    TDS_TRY(make_map(&x->tmB.a_hi, mx.ut_hi, Rp, Mp, kBM));
    TDS_TRY(make_map(&x->tmB.a_lo, mx.ut_lo, Rp, Mp, kBM));
    TDS_TRY(make_map(&x->tmB.b_hi, mx.wt_hi, Rp, (uint64_t)Jm * Mp, kBNB));
    TDS_TRY(make_map(&x->tmB.b_lo, mx.wt_lo, Rp, (uint64_t)Jm * Mp, kBNB));
    TDS_TRY(make_map_f32(&x->te.d, x->d32, Mp, R));
    TDS_TRY(make_map_f32(&x->te.g, mx.g32, Mp, R));
    static bool attr_done = false;
    if (!attr_done) {
        TDS_CUDA(cudaFuncSetAttribute(k_stageA_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kPSmem));
        TDS_CUDA(cudaFuncSetAttribute(k_stageA_tc1, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kRSmem));
        TDS_CUDA(cudaFuncSetAttribute(k_stageB_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kQSmem));
        attr_done = true;
    }
    TDS_CUDA(cudaDeviceSynchronize());
    return autotune(c);
}

int mixed_tuning(tdscha_ctx *c, int *one_acc, int *nsplit, double *ms) {
    MixedExtra *x = extra(c);
    if (!x) { set_error("ctx_tuning: context created without the mixed path"); return TDSCHA_ERR_STATE; }
    *one_acc = x->one_acc;
    *nsplit = c->mx.nsplit;
    *ms = x->tuned_ms;
    return TDSCHA_OK;
}

int mixed_release(tdscha_ctx *c) {
    MixedStore &mx = c->mx;
    void *bufs[] = {mx.d_hi, mx.d_lo, mx.g32, mx.ut_hi, mx.ut_lo, mx.ut32, mx.ft32, mx.wt_hi,
                    mx.wt_lo, mx.y1_hi, mx.y1_lo, mx.qp, mx.gpart};
    for (void *p : bufs)
        cached_free(p);
    if (MixedExtra *x = extra(c)) {
        void *xb[] = {x->sd, x->fmx, x->su, x->sw, x->tcol, x->vs, x->vt, x->absmax, x->d32,
                      x->abcc, x->fpart, x->y1df};
        for (void *p : xb)
            cached_free(p);
        delete x;
    }
    if (mx.err_flag) cudaFreeHost(mx.err_flag);
    mx = MixedStore();
    return TDSCHA_OK;
}

int mixed_check_error(tdscha_ctx *c) {
    if (c->mx.err_flag && *(volatile int *)c->mx.err_flag) {
        int v = *(volatile int *)c->mx.err_flag;
        *(volatile int *)c->mx.err_flag = 0;
        set_error("tensor-core pipeline: a bounded wait expired (code %d)", v);
        return TDSCHA_ERR_TIMEOUT;
    }
    return TDSCHA_OK;
}

static int perturb_mixed_src(tdscha_ctx *c, int apply_d4, const Y1FromPsi *psrc, int nsrc,
                             cudaStream_t st);

int perturb_mixed(tdscha_ctx *c, int apply_d4, cudaStream_t st) {
    return perturb_mixed_src(c, apply_d4, nullptr, 1, st);
}

int perturb_mixed_psi(tdscha_ctx *c, int apply_d4, const double *psi, const double *cty,
                      const double *ctra, cudaStream_t st) {
    Y1FromPsi src{psi, cty, ctra, c->M, c->H, c->ignore_v3};
    return perturb_mixed_src(c, apply_d4, &src, 1, st);
}

int perturb_mixed_pair(tdscha_ctx *c, int apply_d4, const double *psi_a, const double *psi_b,
                       const double *cty, const double *ctra, cudaStream_t st) {
    Y1FromPsi src[2] = {{psi_a, nullptr, nullptr, c->M, c->H, c->ignore_v3},
                        {psi_b, cty, ctra, c->M, c->H, c->ignore_v3}};
    return perturb_mixed_src(c, apply_d4, src, 2, st);
}

// One tensor-core call for nsrc perturbations (1, or 2: the L and L^T
// applications of a bi-Lanczos step) with J symmetry images each: the images
// of perturbation s are s*J .. s*J + J - 1 in every per-call buffer, so stage A
// reads the ensemble once for all of them and every other kernel runs once over
// all images.  Each image has its own W scales, so the results of a
// two-perturbation call are those of two one-perturbation calls, bit for bit.
// psrc == nullptr: one perturbation from the Y1 and R1 buffers.
static int perturb_mixed_src(tdscha_ctx *c, int apply_d4, const Y1FromPsi *psrc, int nsrc,
                             cudaStream_t st) {
    MixedStore &mx = c->mx;
    MixedExtra *x = extra(c);
    if (!x) { set_error("mixed store not prepared"); return TDSCHA_ERR_STATE; }
    const int M = c->M, Mp = mx.Mp, J = c->J;
    const int Jb = nsrc * J;   // images in this call
    if (Jb > x->jmax || (nsrc > 1 && !psrc)) { set_error("mixed call: bad perturbation count"); return TDSCHA_ERR_ARG; }
    const long R = c->Nrows, Rp = mx.Rp;
    const int ntBb = (int)ceil_div((long)Jb * Mp, kBNB), ldGb = ntBb * kBNB;
    int *err_dev = nullptr;
    TDS_CUDA(cudaHostGetDevicePointer((void **)&err_dev, mx.err_flag, 0));
    {
        // the Y1 limbs, epilogue vectors and W-scale maxima of every
        // perturbation of the call, perturbation s at image offset s * J
        ProfScope ps(c, 5, st);
        if (J > 1) {
            const size_t sm = sizeof(float) * Mp;
            const dim3 gy(M, nsrc), gi(J * Mp, nsrc);
            if (psrc) {
                const SrcPair<Y1FromPsi> sp{{psrc[0], psrc[nsrc - 1]}};
                TDS_CUDA(launch_pdl(k_y1_df<Y1FromPsi>, gy, 256, 0, st, sp, M, x->y1df));
                TDS_CUDA(launch_pdl(k_prep_y1_img<Y1FromPsi>, gi, 256, sm, st, sp,
                                    (const float2 *)x->y1df, c->sc_idx, c->sc_val, c->sc_val2,
                                    c->maxdeg, c->fY, c->fpsi, x->sd, M, Mp, mx.y1_hi, mx.y1_lo,
                                    x->tcol, x->vs, x->vt, x->absmax));
            } else {
                const Y1FromBuffers b1{c->Y1, c->R1, M};
                const SrcPair<Y1FromBuffers> sp{{b1, b1}};
                TDS_CUDA(launch_pdl(k_y1_df<Y1FromBuffers>, gy, 256, 0, st, sp, M, x->y1df));
                TDS_CUDA(launch_pdl(k_prep_y1_img<Y1FromBuffers>, gi, 256, sm, st, sp,
                                    (const float2 *)x->y1df, c->sc_idx, c->sc_val, c->sc_val2,
                                    c->maxdeg, c->fY, c->fpsi, x->sd, M, Mp, mx.y1_hi, mx.y1_lo,
                                    x->tcol, x->vs, x->vt, x->absmax));
            }
        } else {
            const dim3 g(Mp, nsrc);
            if (psrc) {
                const SrcPair<Y1FromPsi> sp{{psrc[0], psrc[nsrc - 1]}};
                TDS_CUDA(launch_pdl(k_prep_y1<Y1FromPsi>, g, 256, 0, st, sp, c->fY, c->fpsi, x->sd,
                                    M, Mp, mx.y1_hi, mx.y1_lo, x->tcol, x->vs, x->vt, x->absmax));
            } else {
                const Y1FromBuffers b1{c->Y1, c->R1, M};
                const SrcPair<Y1FromBuffers> sp{{b1, b1}};
                TDS_CUDA(launch_pdl(k_prep_y1<Y1FromBuffers>, g, 256, 0, st, sp, c->fY, c->fpsi,
                                    x->sd, M, Mp, mx.y1_hi, mx.y1_lo, x->tcol, x->vs, x->vt,
                                    x->absmax));
            }
        }
    }
    StageAArgs ga{};
    ga.R = R;
    ga.Mp = Mp;
    ga.nkb = Mp / kPBK;
    ga.nct = mx.nctile;
    ga.J = Jb;
    ga.b_box = x->bnA;
    ga.ntiles = (long)ceil_div(R, kBM) * Jb * mx.nctile;
    ga.tcol = x->tcol;
    ga.vec_s = x->vs;
    ga.vec_t = x->vt;
    ga.qpst = mx.qp;
    ga.err = err_dev;
    ga.budget = x->budget;
    {
        ProfScope ps(c, 0, st);
        int grid = (int)std::min<long>(ga.ntiles, x->nsm);
        if (x->one_acc)
            TDS_CUDA(launch_pdl(k_stageA_tc1, grid, 192, kRSmem, st, x->tmA1, x->te, ga));
        else
            TDS_CUDA(launch_pdl(k_stageA_tc, grid, 192, kPSmem, st, x->tmA, x->te, ga));
    }
    {
        ProfScope ps(c, 1, st);
        TDS_CUDA(launch_pdl(k_rows_mixed, dim3(ceil_div(R, 128), Jb), 128, 0, st, mx.qp,
                            mx.nctile, R, c->rho_div, c->rho, apply_d4, x->abcc, x->absmax));
    }
    {
        ProfScope ps(c, 2, st);
        if (J == 1) {
            dim3 g(ceil_div(M, kWRows), x->nfchunk);
            TDS_CUDA(launch_pdl(k_wbuild_pair, g, 256, 0, st, mx.ft32, mx.ut32, x->abcc,
                                x->absmax, x->fmx, x->su, R, Rp, M, Mp, Jb, mx.wt_hi, mx.wt_lo,
                                x->sw, x->fpart));
        } else {
            dim3 g(ceil_div(M, kWRows), x->nfchunk, Jb);
            TDS_CUDA(launch_pdl(k_wbuild_img, g, 256, 0, st, mx.ft32, mx.ut32, x->abcc,
                                x->absmax, x->fmx, x->su, R, Rp, M, Mp, mx.wt_hi, mx.wt_lo, x->sw,
                                x->fpart));
        }
    }
    StageBArgs gb{};
    gb.nkb = x->kbps;
    gb.nkb_total = x->nkbB;
    gb.Mp = Mp;
    gb.ldG = x->ldG;
    gb.ntile = x->ntB;
    gb.ntile_b = ntBb;
    gb.ldGb = ldGb;
    gb.JMp = Jb * Mp;
    gb.nitems = (long)x->ntB * ntBb * mx.nsplit;
    gb.su = x->su;
    gb.sw = x->sw;
    gb.gpart = mx.gpart;
    gb.err = err_dev;
    gb.budget = x->budget;
    {
        ProfScope ps(c, 3, st);
        int grid = (int)std::min<long>(gb.nitems, x->nsm);
        TDS_CUDA(launch_pdl(k_stageB_tc, grid, 192, kQSmem, st, x->tmB, gb));
    }
    const long sstride = (long)x->ldG * ldGb;
    if (J > 1) {
        for (int sidx = 0; sidx < nsrc; ++sidx) {
            const long io = (long)sidx * J;
            TDS_TRY(psi_finalize32(c, mx.gpart + io * Mp, mx.nsplit, sstride, Mp, ldGb,
                                   x->fpart + io * x->nfchunk * M, x->nfchunk,
                                   sidx ? c->f2 : c->f, sidx ? c->d2v2 : c->d2v, st));
        }
    } else {
        // both perturbations' split-K sums and (f, d2v) in one launch
        ProfScope ps(c, 4, st);
        const int nt = ceil_div(M, 32);
        TDS_CUDA(launch_pdl(k_gfinal, dim3(4 * (nt * (nt + 1) / 2), nsrc), 256, 0, st, mx.gpart,
                            mx.nsplit, (long)ldGb, sstride, M, Mp, x->fpart, x->nfchunk,
                            c->sum_rho * c->S, c->f, c->d2v, c->f2, c->d2v2));
    }
    return TDSCHA_OK;
}

}  // namespace tdscha

// wp_gemm.cu -- BF16 GEMM on the fifth-generation tensor cores (sm_103a):
//
//     C[M][N] = epilogue( A[M][K] . B[N][K]^T + bias[N] )
//
// with A and B row-major BF16 (both K-major), FP32 accumulation in tensor
// memory, and an epilogue that adds the bias, optionally applies GELU (and
// keeps the pre-activation), and stores BF16 or FP32.  This is the building
// block of the learned proposal network (forward layers, and with
// transposed operands its backward products).
//
// A persistent CTA per SM walks 128 x 256 output tiles with 6 warps:
//   warp 0 (one thread)  TMA producer: 64-wide K slices of A and B into a
//                        4-stage shared-memory ring (128-byte swizzle),
//                        signalled on the stage's `full` mbarrier;
//   warp 1 (one thread)  MMA issuer: four tcgen05.mma (M128 N256 K16) per
//                        stage into one of two 256-column TMEM accumulators,
//                        tcgen05.commit onto the stage's `empty` mbarrier so
//                        the producer can refill it, and onto the
//                        accumulator's `full` mbarrier after the last K
//                        slice; warp 1 also owns the TMEM allocation;
//   warps 2-5            epilogue: each reads its 32 TMEM lanes (rows) in
//                        32-column chunks with tcgen05.ld, stages them in
//                        shared memory, stores rows contiguously, and frees
//                        the accumulator (its `empty` mbarrier) for the
//                        tile after next.
// Every mbarrier wait is bounded; on expiry the CTA records an error code,
// stops issuing work, waits (bounded) for what it issued and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#define GEMM_BM 128
#define GEMM_BN 256
#define GEMM_BK 64
#define GEMM_STAGES 4
#define GEMM_THREADS 192
#define GEMM_TMEM_COLS 256
#define GEMM_A_STAGE (GEMM_BM * GEMM_BK * 2)  // 16 KB
#define GEMM_B_STAGE (GEMM_BN * GEMM_BK * 2)  // 32 KB
#define GEMM_WAIT_LIMIT (1L << 22)
#define GEMM_SROW 36  // floats per row of the epilogue staging tile (32 + 4: conflict-free float4)

typedef __nv_bfloat16 bf16_t;

struct GemmParams {
    int M, N, K;
    void* C;            // [M][ldc] BF16 or FP32
    int ldc;
    int c_fp32;         // 1: FP32 output, 0: BF16
    const float* bias;  // [N] or null
    int act;            // 0 none, 1 GELU (erf form)
    __nv_bfloat16* Z;   // pre-activation [M][ldc] BF16, or null
    int accumulate;     // unused (must be 0)
    int* err;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
    return ok != 0;
}

// Bounded wait for the phase of `parity`; false (and an error code) when
// the limit expires.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
    for (long i = 0; i < GEMM_WAIT_LIMIT; i++)
        if (mbar_try_wait(bar, parity)) return true;
    atomicExch(err, code);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
            ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
            : "memory");
}

// Shared-memory matrix descriptor of a K-major tile written by TMA with the
// 128-byte swizzle: rows of 128 B, 8-row atoms 1024 B apart (stride byte
// offset), fixed field 0b001 at bit 46, swizzle mode 2 (128 B) at bit 61.
// The leading byte offset is unused for this layout.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and
// B BF16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t gemm_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "setp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
            "}\n" ::"r"(tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
            : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
    asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
            "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
            "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
              "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
              "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ float gelu_erf(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Persistent: CTA b takes tiles b, b + gridDim.x, ... (M blocks fastest, so
// the CTAs running at once share B tiles in L2).  Two TMEM accumulators
// (2 x 256 columns): the MMA thread fills one while the epilogue warps drain
// the other.  Epilogue stores go through a per-warp shared-memory tile so
// that global stores are row-contiguous.
__global__ void __launch_bounds__(GEMM_THREADS, 1)
        wp_gemm_tn_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                          GemmParams p) {
    extern __shared__ uint8_t gemm_smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(gemm_smem_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = smem;
    uint8_t* sB = smem + GEMM_STAGES * GEMM_A_STAGE;
    float* stage_out = reinterpret_cast<float*>(sB + GEMM_STAGES * GEMM_B_STAGE);  // [4 warps][32][GEMM_SROW]
    uint64_t* full = reinterpret_cast<uint64_t*>(stage_out + 4 * 32 * GEMM_SROW);
    uint64_t* empty = full + GEMM_STAGES;
    uint64_t* acc_full = empty + GEMM_STAGES;  // [2]
    uint64_t* acc_empty = acc_full + 2;        // [2]
    uint64_t* done = acc_empty + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nk = p.K / GEMM_BK;
    const int mblocks = (p.M + GEMM_BM - 1) / GEMM_BM;
    const int nblocks = (p.N + GEMM_BN - 1) / GEMM_BN;
    const int ntiles = mblocks * nblocks;

    if (threadIdx.x == 0) {
        for (int s = 0; s < GEMM_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * GEMM_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // TMA producer over every (tile, k) of this CTA
            int it = 0;
            for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
                const int m0 = (t % mblocks) * GEMM_BM, n0 = (t / mblocks) * GEMM_BN;
                for (int kt = 0; kt < nk; kt++, it++) {
                    const int s = it % GEMM_STAGES, round = it / GEMM_STAGES;
                    if (*abort_flag || !mbar_wait(&empty[s], (round & 1) ^ 1, p.err, 101)) {
                        *abort_flag = 1;
                        break;
                    }
                    mbar_expect_tx(&full[s], GEMM_A_STAGE + GEMM_B_STAGE);
                    tma_load_2d(sA + s * GEMM_A_STAGE, &tmA, kt * GEMM_BK, m0, &full[s]);
                    tma_load_2d(sB + s * GEMM_B_STAGE, &tmB, kt * GEMM_BK, n0, &full[s]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            const uint32_t idesc = gemm_idesc(GEMM_BM, GEMM_BN);
            int it = 0, li = 0;
            for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x, li++) {
                const int b = li & 1, use = li >> 1;
                if (!mbar_wait(&acc_empty[b], (use & 1) ^ 1, p.err, 105)) {
                    *abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc = tmem + (uint32_t)(b * GEMM_TMEM_COLS);
                bool ok = true;
                for (int kt = 0; kt < nk; kt++, it++) {
                    const int s = it % GEMM_STAGES, round = it / GEMM_STAGES;
                    if (*abort_flag || !mbar_wait(&full[s], round & 1, p.err, 102)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a0 = smem_u32(sA + s * GEMM_A_STAGE), b0 = smem_u32(sB + s * GEMM_B_STAGE);
#pragma unroll
                    for (int k = 0; k < GEMM_BK / 16; k++)
                        mma_bf16(acc, sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), idesc, (kt | k) != 0 ? 1u : 0u);
                    mma_commit(&empty[s]);
                }
                if (!ok) {
                    *abort_flag = 1;
                    break;
                }
                mma_commit(&acc_full[b]);
            }
            mma_commit(done);  // every MMA this thread issued has completed when this arrives
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31
        const int q = warp & 3;
        float* st = stage_out + q * 32 * GEMM_SROW;
        int li = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, li++) {
            const int b = li & 1, use = li >> 1;
            const int m0 = (t % mblocks) * GEMM_BM, n0 = (t / mblocks) * GEMM_BN;
            if (*abort_flag || !mbar_wait(&acc_full[b], use & 1, p.err, 103)) {
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int rbase = m0 + 32 * q;
            for (int ch = 0; ch < GEMM_BN / 32; ch++) {
                uint32_t r[32];
                tmem_ld32(tmem + (uint32_t)(b * GEMM_TMEM_COLS) + ((uint32_t)(32 * q) << 16) + (uint32_t)(ch * 32), r);
                const int c0 = n0 + ch * 32;
                if (c0 >= p.N || rbase >= p.M) continue;  // warp-uniform
                float v[32];
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    float x = __uint_as_float(r[j]);
                    if (p.bias) x += (c0 + j < p.N) ? p.bias[c0 + j] : 0.0f;
                    v[j] = x;
                }
                // two passes through the staging tile: pre-activation, output
                for (int pass = p.Z ? 0 : 1; pass < 2; pass++) {
                    float o[32];
#pragma unroll
                    for (int j = 0; j < 32; j++) o[j] = (pass == 1 && p.act == 1) ? gelu_erf(v[j]) : v[j];
                    const bool f32 = pass == 1 && p.c_fp32;
                    __syncwarp();
                    if (f32) {
#pragma unroll
                        for (int j = 0; j < 32; j += 4)
                            *reinterpret_cast<float4*>(st + lane * GEMM_SROW + j) = make_float4(o[j], o[j + 1], o[j + 2], o[j + 3]);
                    } else {
                        uint32_t* su = reinterpret_cast<uint32_t*>(st + lane * GEMM_SROW);
#pragma unroll
                        for (int j = 0; j < 16; j += 4) {
                            uint4 u;
                            __nv_bfloat162 h0 = __floats2bfloat162_rn(o[2 * j], o[2 * j + 1]);
                            __nv_bfloat162 h1 = __floats2bfloat162_rn(o[2 * j + 2], o[2 * j + 3]);
                            __nv_bfloat162 h2 = __floats2bfloat162_rn(o[2 * j + 4], o[2 * j + 5]);
                            __nv_bfloat162 h3 = __floats2bfloat162_rn(o[2 * j + 6], o[2 * j + 7]);
                            u.x = *reinterpret_cast<uint32_t*>(&h0);
                            u.y = *reinterpret_cast<uint32_t*>(&h1);
                            u.z = *reinterpret_cast<uint32_t*>(&h2);
                            u.w = *reinterpret_cast<uint32_t*>(&h3);
                            *reinterpret_cast<uint4*>(su + j) = u;
                        }
                    }
                    __syncwarp();
                    // row-contiguous stores: FP32 rows are 8 x 16 B (8 lanes
                    // per row, 4 rows per pass), BF16 rows 4 x 16 B
                    const bool full_cols = c0 + 32 <= p.N;
                    if (f32) {
                        float* C = reinterpret_cast<float*>(p.C);
                        for (int i = 0; i < 8; i++) {
                            const int rr = i * 4 + (lane >> 3), cc = (lane & 7) * 4;
                            const int row = rbase + rr;
                            if (row >= p.M) continue;
                            const float4 val = *reinterpret_cast<const float4*>(st + rr * GEMM_SROW + cc);
                            float* dst = C + (long)row * p.ldc + c0 + cc;
                            if (full_cols && (p.ldc & 3) == 0) {
                                *reinterpret_cast<float4*>(dst) = val;
                            } else {
                                const float e4[4] = {val.x, val.y, val.z, val.w};
                                for (int j = 0; j < 4; j++)
                                    if (c0 + cc + j < p.N) dst[j] = e4[j];
                            }
                        }
                    } else {
                        bf16_t* D = pass == 0 ? p.Z : reinterpret_cast<bf16_t*>(p.C);
                        const uint32_t* su = reinterpret_cast<const uint32_t*>(st);
                        for (int i = 0; i < 4; i++) {
                            const int rr = i * 8 + (lane >> 2), cw = (lane & 3) * 4;  // 4 words = 8 BF16
                            const int row = rbase + rr;
                            if (row >= p.M) continue;
                            const uint4 val = *reinterpret_cast<const uint4*>(su + rr * GEMM_SROW + cw);
                            bf16_t* dst = D + (long)row * p.ldc + c0 + 2 * cw;
                            if (full_cols && (p.ldc & 7) == 0) {
                                *reinterpret_cast<uint4*>(dst) = val;
                            } else {
                                const uint32_t w4[4] = {val.x, val.y, val.z, val.w};
                                for (int j = 0; j < 8; j++)
                                    if (c0 + 2 * cw + j < p.N) {
                                        const uint32_t wv = w4[j >> 1];
                                        const unsigned short hv = (j & 1) ? (unsigned short)(wv >> 16) : (unsigned short)(wv & 0xffffu);
                                        dst[j] = __ushort_as_bfloat16(hv);
                                    }
                            }
                        }
                    }
                }
            }
            // this accumulator may be refilled
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        // free the columns only after every issued MMA has completed
        mbar_wait(done, 0, p.err, 104);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * GEMM_TMEM_COLS)
                     : "memory");
    }
}

// ------------------------------------------------------------------ host
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                    cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(f);
    }
    return fn;
}

// Row-major BF16 [rows][K] (row pitch ld elements), boxes of 64 x box_rows.
static bool make_map(CUtensorMap* map, const void* ptr, int rows, int K, int ld, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {GEMM_BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t wp_gemm_smem_bytes() {
    return 1024 + GEMM_STAGES * (GEMM_A_STAGE + GEMM_B_STAGE) + 4 * 32 * GEMM_SROW * 4 + (2 * GEMM_STAGES + 5) * 8 + 16;
}

// C = act(A . B^T + bias).  A: [M][K] (pitch lda), B: [N][K] (pitch ldb),
// both BF16 row-major, 16-byte aligned, K a multiple of 64, pitches
// multiples of 8 elements.  Returns cudaErrorInvalidValue on a shape the
// kernel does not take.
cudaError_t wp_gemm_bf16_tn(const void* A, int lda, const void* B, int ldb, int M, int N, int K, void* C, int ldc,
                            int c_fp32, const float* bias, int act, void* Z, int accumulate, int* err,
                            cudaStream_t s) {
    if (M <= 0 || N <= 0 || K <= 0 || K % GEMM_BK != 0 || lda % 8 || ldb % 8 || lda < K || ldb < K || ldc < N ||
        ((uintptr_t)A & 15) || ((uintptr_t)B & 15) || accumulate)
        return cudaErrorInvalidValue;
    CUtensorMap ma, mb;
    if (!make_map(&ma, A, M, K, lda, GEMM_BM) || !make_map(&mb, B, N, K, ldb, GEMM_BN)) return cudaErrorInvalidValue;
    GemmParams p;
    p.M = M;
    p.N = N;
    p.K = K;
    p.C = C;
    p.ldc = ldc;
    p.c_fp32 = c_fp32;
    p.bias = bias;
    p.act = act;
    p.Z = reinterpret_cast<__nv_bfloat16*>(Z);
    p.accumulate = accumulate;
    p.err = err;
    const size_t smem = wp_gemm_smem_bytes();
    cudaFuncSetAttribute(wp_gemm_tn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    static int sms[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && sms[dev] == 0) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    const int tiles = ((M + GEMM_BM - 1) / GEMM_BM) * ((N + GEMM_BN - 1) / GEMM_BN);
    const int grid = std::min(tiles, (dev >= 0 && dev < 64 && sms[dev] > 0) ? sms[dev] : 148);
    wp_gemm_tn_kernel<<<grid, GEMM_THREADS, smem, s>>>(ma, mb, p);
    return cudaGetLastError();
}

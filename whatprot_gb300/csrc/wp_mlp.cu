// wp_mlp.cu -- the learned proposal network: an MLP from a radiometry
// (T*C intensities, zero-padded to 64) to logits over the peptide set,
//
//     x -> GELU(W1 x + b1) -> GELU(W2 h1 + b2) -> W3 h2 + b3     (1024 wide)
//
// with BF16 weights and activations and FP32 accumulation on the tensor
// cores (wp_gemm.cu), trained with softmax cross-entropy and Adam on reads
// simulated on the GPU (wp_sim.cu), used to propose the top-H peptides that
// the HMM then rescores, in place of the kNN stage of the hybrid classifier.
// The reference has no such network; this file has no reference
// counterpart.
//
// All products are C = A . B^T with K-major operands (wp_gemm_bf16_tn), so
// the backward pass keeps transposed BF16 copies where an operand's
// reduction dimension would otherwise be strided:
//     dH2 = dL . W3         uses W3^T  [1024][P]
//     dW3 = dL^T . H2       uses dL^T [P][B] and H2^T [1024][B]
//     dH1 = dZ2 . W2        uses W2^T
//     dW2 = dZ2^T . H1      uses dZ2^T, H1^T
//     dW1 = dZ1^T . X       uses dZ1^T, X^T
// Master weights, gradients and Adam moments are FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <curand_kernel.h>
#include <math.h>
#include <stdint.h>

typedef __nv_bfloat16 bf16;

// Radiometries (FP32 or FP64, [B][TC]) to BF16 inputs [B][64] (zero padded).
__global__ void wp_mlp_input_kernel(const float* __restrict__ xf, const double* __restrict__ xd, int B, int TC,
                                    bf16* __restrict__ X) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)B * 64) return;
    const long b = i / 64;
    const int d = (int)(i % 64);
    float v = 0.f;
    if (d < TC) v = xf ? xf[b * TC + d] : (float)xd[b * TC + d];
    X[i] = __float2bfloat16_rn(v);
}

// out[c][r] = in[r][c] for a rows x cols BF16 matrix (pitches in elements).
__global__ void wp_transpose_bf16_kernel(const bf16* __restrict__ in, int rows, int cols, int ld_in,
                                         bf16* __restrict__ out, int ld_out) {
    __shared__ unsigned short tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        tile[j][threadIdx.x] = (r < rows && c < cols) ? __bfloat16_as_ushort(in[(long)r * ld_in + c]) : 0;
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = c0 + j, r = r0 + threadIdx.x;
        if (c < cols && r < rows) out[(long)c * ld_out + r] = __ushort_as_bfloat16(tile[threadIdx.x][j]);
    }
}

// Block-wide reductions in a fixed order (warp trees, then warp 0).
__device__ float block_max(float v, float* sh) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? sh[l] : -INFINITY;
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (l == 0) sh[0] = v;
    }
    __syncthreads();
    return sh[0];
}

__device__ float block_sum(float v, float* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (l == 0) sh[0] = v;
    }
    __syncthreads();
    return sh[0];
}

// One CTA per row: softmax over the first P logits, cross-entropy against
// the label (rows with label < 0 are skipped: loss 0, gradient 0), and the
// logit gradient (softmax - onehot) * scale as BF16 (zero past P).
__global__ void wp_softmax_ce_kernel(const float* __restrict__ logits, int P, int ld, const int* __restrict__ labels,
                                     float scale, bf16* __restrict__ dL, double* __restrict__ loss) {
    __shared__ float sh[32];
    const long row = blockIdx.x;
    const float* l = logits + row * ld;
    const int y = labels[row];
    float mx = -INFINITY;
    for (int j = threadIdx.x; j < P; j += blockDim.x) mx = fmaxf(mx, l[j]);
    mx = block_max(mx, sh);
    float s = 0.f;
    for (int j = threadIdx.x; j < P; j += blockDim.x) s += expf(l[j] - mx);
    s = block_sum(s, sh);
    const float inv = 1.0f / s;
    bf16* g = dL + row * ld;
    for (int j = threadIdx.x; j < ld; j += blockDim.x) {
        float v = 0.f;
        if (y >= 0 && j < P) v = (expf(l[j] - mx) * inv - (j == y ? 1.f : 0.f)) * scale;
        g[j] = __float2bfloat16_rn(v);
    }
    if (threadIdx.x == 0) loss[row] = y >= 0 ? (double)(logf(s) + mx - l[y]) : 0.0;
}

// dZ = dH * GELU'(Z), GELU(z) = z Phi(z):  GELU'(z) = Phi(z) + z phi(z).
__global__ void wp_gelu_bwd_kernel(const float* __restrict__ dH, const bf16* __restrict__ Z, long n,
                                   bf16* __restrict__ dZ) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float z = __bfloat162float(Z[i]);
    const float d = 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
    dZ[i] = __float2bfloat16_rn(dH[i] * d);
}

// Column sums of a BF16 [rows][ld] matrix, one thread per column, rows in
// order (deterministic).
__global__ void wp_colsum_bf16_kernel(const bf16* __restrict__ M, int rows, int cols, int ld, float* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.f;
    for (int r = 0; r < rows; r++) s += __bfloat162float(M[(long)r * ld + c]);
    out[c] = s;
}

// Adam (Kingma & Ba 2015) on FP32 master weights; refreshes the BF16 copy.
__global__ void wp_adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                               float* __restrict__ v, long n, float lr, float b1, float b2, float eps, float bc1,
                               float bc2, bf16* __restrict__ wb) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16_rn(wi);
}

__global__ void wp_f32_to_bf16_kernel(const float* __restrict__ in, long n, bf16* __restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2bfloat16_rn(in[i]);
}

// Gaussian initialisation N(0, std^2) of rows [0, valid_rows) of a
// [rows][cols] matrix (others zero), Philox stream per element.
__global__ void wp_init_normal_kernel(float* __restrict__ w, long rows, long cols, long valid_rows, float std,
                                      unsigned long long seed) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    if (i / cols >= valid_rows) {
        w[i] = 0.f;
        return;
    }
    curandStatePhilox4_32_10_t st;
    curand_init(seed, (unsigned long long)i, 0ull, &st);
    w[i] = std * curand_normal(&st);
}

// Sortable unsigned key of a float (ascending order of the floats).
__device__ __forceinline__ unsigned fkey(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// The exact fallback of the top-h selection, one CTA (256 threads) per read
// of the list rows[0 .. *nrows) (persistent over it): the h largest of the
// first P logits by (logit, index), by radix select on the sortable keys,
// then sorted ascending; writes peptide indices and softmax probabilities,
// and the sum of probability x peptide count over the candidates.
__global__ void wp_topk_kernel(const float* __restrict__ logits, int P, int ld, int h, const int* __restrict__ counts,
                               int* __restrict__ out_idx, float* __restrict__ out_prob, double* __restrict__ out_mass,
                               const int* __restrict__ rows, const int* __restrict__ nrows) {
    __shared__ unsigned hist[256];
    __shared__ float sh[32];
    __shared__ unsigned long long skey[1024];
    __shared__ int sidx[1024];
    __shared__ int nsel;
  for (int it = blockIdx.x; it < *nrows; it += gridDim.x) {
    const long row = rows[it];
    const float* l = logits + row * ld;
    // softmax normaliser
    float mx = -INFINITY;
    for (int j = threadIdx.x; j < P; j += blockDim.x) mx = fmaxf(mx, l[j]);
    mx = block_max(mx, sh);
    float s = 0.f;
    for (int j = threadIdx.x; j < P; j += blockDim.x) s += expf(l[j] - mx);
    s = block_sum(s, sh);
    // radix select of the h-th largest key (count based, from the top)
    unsigned prefix = 0u, mask = 0u;
    int want = min(h, P);
    for (int pass = 0; pass < 4; pass++) {
        const int shift = 24 - 8 * pass;
        for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0u;
        __syncthreads();
        for (int j = threadIdx.x; j < P; j += blockDim.x) {
            const unsigned k = fkey(l[j]);
            if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 255u], 1u);
        }
        __syncthreads();
        __shared__ int sdigit, sbefore;
        if (threadIdx.x == 0) {
            int c = 0, d = 255;
            for (; d > 0; d--) {
                if (c + (int)hist[d] >= want) break;
                c += (int)hist[d];
            }
            sdigit = d;
            sbefore = c;
        }
        __syncthreads();
        prefix |= (unsigned)sdigit << shift;
        mask |= 255u << shift;
        want -= sbefore;
        __syncthreads();
    }
    // keys above the threshold, plus `want` of those equal to it with the
    // largest indices (one thread walks the ties from the top index down)
    if (threadIdx.x == 0) nsel = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < P; j += blockDim.x) {
        const unsigned k = fkey(l[j]);
        if (k > prefix) {
            const int pos = atomicAdd(&nsel, 1);
            skey[pos] = ((unsigned long long)k << 32) | (unsigned)j;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int taken = 0;
        for (int j = P - 1; j >= 0 && taken < want; j--)
            if (fkey(l[j]) == prefix) {
                skey[nsel++] = ((unsigned long long)prefix << 32) | (unsigned)j;
                taken++;
            }
    }
    __syncthreads();
    const int n = nsel;
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int i = n + threadIdx.x; i < n2; i += blockDim.x) skey[i] = ~0ull;
    __syncthreads();
    for (int size = 2; size <= n2; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0;
                    const unsigned long long a = skey[i], b = skey[j];
                    if ((a > b) == up) {
                        skey[i] = b;
                        skey[j] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int j = (int)(skey[i] & 0xffffffffu);
        out_idx[row * h + i] = j;
        out_prob[row * h + i] = expf(l[j] - mx) / s;
        sidx[i] = j;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double mass = 0.0;
        for (int i = 0; i < n; i++) mass += (double)(expf(l[sidx[i]] - mx) / s) * (double)counts[sidx[i]];
        out_mass[row] = mass;
    }
    __syncthreads();
  }
}

// The top-h selection, one warp per read (persistent over the reads): a
// sample of TK_SAMPLE logits at a fixed stride gives, by a bitwise search
// for its order statistic, a threshold that about 2 h of the read's logits
// reach; one pass over the logits
// keeps those at or above it (composite key: sortable logit bits, then the
// index) in the warp's shared buffer and forms the softmax normaliser
// online; the buffer, sorted, yields the h largest, written ascending as the
// fallback kernel does.  A read whose kept set is smaller than h or larger
// than the buffer goes to fail_rows for the exact fallback kernel.
#define TK_WARPS 8
#define TK_CAP 1024
#define TK_SAMPLE 1024

// Bitonic sort, descending, of buf[0 .. n) (n a power of two) by one warp.
__device__ __forceinline__ void tk_warp_sort_desc(unsigned long long* buf, int n) {
    const int lane = threadIdx.x & 31;
    for (int size = 2; size <= n; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = lane; i < n; i += 32) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool desc = (i & size) == 0;
                    const unsigned long long a = buf[i], b = buf[j];
                    if ((a < b) == desc) {
                        buf[i] = b;
                        buf[j] = a;
                    }
                }
            }
            __syncwarp();
        }
}

__global__ void __launch_bounds__(TK_WARPS * 32) wp_topk_warp_kernel(const float* __restrict__ logits, int R, int P,
                                                                      int ld, int h, const int* __restrict__ counts,
                                                                      int* __restrict__ out_idx,
                                                                      float* __restrict__ out_prob,
                                                                      double* __restrict__ out_mass,
                                                                      int* __restrict__ fail_rows,
                                                                      int* __restrict__ fail_count, int vec4) {
    extern __shared__ unsigned long long tk_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long* buf = tk_smem + (size_t)warp * TK_CAP;
    unsigned* hist = reinterpret_cast<unsigned*>(tk_smem + (size_t)TK_WARPS * TK_CAP) + warp * 256;
    const unsigned lt = (1u << lane) - 1u;
    for (long row = (long)blockIdx.x * TK_WARPS + warp; row < R; row += (long)gridDim.x * TK_WARPS) {
        const float* l = logits + row * ld;
        // threshold: the composite key that about 2.5 h logits reach
        unsigned long long tau = 0ull;
        if (P > TK_CAP) {
            // the rank-th largest sample key, bit by bit from the top: the
            // largest t with at least `rank` sample keys >= t
            // TK_SAMPLE / 4 blocks of four neighbouring logits at a fixed
            // stride (one 16-byte load each)
            unsigned sk[TK_SAMPLE / 32];
#pragma unroll
            for (int u = 0; u < TK_SAMPLE / 128; u++) {
                const int b = u * 32 + lane;
                int j = (int)(((long)b * P) / (TK_SAMPLE / 4)) & ~3;
                j = min(j, (P - 4) & ~3);  // a multiple of 4 (16-byte aligned), j + 3 < P
                float4 v;
                if (vec4) {
                    v = *reinterpret_cast<const float4*>(l + j);
                } else {
                    v = make_float4(l[j], l[j + 1], l[j + 2], l[j + 3]);
                }
                sk[4 * u] = fkey(v.x);
                sk[4 * u + 1] = fkey(v.y);
                sk[4 * u + 2] = fkey(v.z);
                sk[4 * u + 3] = fkey(v.w);
            }
            const int rank = min(TK_SAMPLE, (int)ceilf(2.0f * (float)h * (float)TK_SAMPLE / (float)P) + 4);
            unsigned t = 0u;
#pragma unroll 1
            for (int bit = 31; bit >= 0; bit--) {
                const unsigned cand = t | (1u << bit);
                int c = 0;
#pragma unroll
                for (int u = 0; u < TK_SAMPLE / 32; u++) c += sk[u] >= cand ? 1 : 0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
                if (c >= rank) t = cand;
            }
            tau = (unsigned long long)t << 32;  // every index of a key at the threshold
        }
        // the float at the threshold key: x >= tf keeps every key >= tau
        // (and possibly -0.0 at +0.0, harmless: extra keys are sorted out)
        const unsigned th = (unsigned)(tau >> 32);
        const float tf = P > TK_CAP ? __uint_as_float((th & 0x80000000u) ? (th & 0x7fffffffu) : ~th) : -INFINITY;
        // one pass: keep keys >= tau; online max and sum of exp
        int cnt = 0;
        float m = -INFINITY, sum = 0.0f;
        // element j: online softmax, then kept when its key reaches tau
        // (the normaliser uses the fast exponential: relative error near
        // 1e-6 over the logit range; the probabilities written use expf)
        auto visit = [&](int j, float x, bool in) {
            if (in) {
                if (x > m) {
                    sum = sum * __expf(m - x) + 1.0f;
                    m = x;
                } else {
                    sum += __expf(x - m);
                }
            }
            const bool keep = in && x >= tf;
            const unsigned ball = __ballot_sync(0xffffffffu, keep);
            if (ball) {
                if (keep) {
                    const int pos = cnt + __popc(ball & lt);
                    if (pos < TK_CAP) buf[pos] = ((unsigned long long)fkey(x) << 32) | (unsigned)j;
                }
                cnt += __popc(ball);
            }
        };
        int j0 = 0;
        if (vec4) {  // 16-byte rows: eight float4 per lane in flight
            // eight independent online-softmax states (one per float4 slot,
            // so the exponentials do not form one long dependent chain),
            // merged below; the kept keys of a 1,024-logit chunk are placed
            // with one warp scan of the lanes' counts (their order in the
            // buffer does not matter: it is sorted)
            const float4* l4 = reinterpret_cast<const float4*>(l);
            float mu[8], su[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                mu[u] = -INFINITY;
                su[u] = 0.0f;
            }
            for (; j0 + 1024 <= P; j0 += 1024) {
                float4 v[8];
#pragma unroll
                for (int u = 0; u < 8; u++) v[u] = l4[(j0 >> 2) + 32 * u + lane];
                unsigned km = 0u;
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const float mx = fmaxf(fmaxf(v[u].x, v[u].y), fmaxf(v[u].z, v[u].w));
                    if (mx > mu[u]) {
                        su[u] = su[u] * __expf(mu[u] - mx);
                        mu[u] = mx;
                    }
                    su[u] += (__expf(v[u].x - mu[u]) + __expf(v[u].y - mu[u])) +
                             (__expf(v[u].z - mu[u]) + __expf(v[u].w - mu[u]));
                    km |= (v[u].x >= tf ? 1u : 0u) << (4 * u);
                    km |= (v[u].y >= tf ? 1u : 0u) << (4 * u + 1);
                    km |= (v[u].z >= tf ? 1u : 0u) << (4 * u + 2);
                    km |= (v[u].w >= tf ? 1u : 0u) << (4 * u + 3);
                }
                const int mine = __popc(km);
                int incl = mine;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                int pos = cnt + incl - mine;
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    unsigned m4 = (km >> (4 * u)) & 15u;
                    while (m4) {
                        const int c = __ffs(m4) - 1;
                        m4 &= m4 - 1;
                        const float x = c == 0 ? v[u].x : c == 1 ? v[u].y : c == 2 ? v[u].z : v[u].w;
                        if (pos < TK_CAP)
                            buf[pos] = ((unsigned long long)fkey(x) << 32) | (unsigned)(j0 + 128 * u + 4 * lane + c);
                        pos++;
                    }
                }
                cnt += __shfl_sync(0xffffffffu, incl, 31);
            }
            // the lane's softmax state from its eight
#pragma unroll
            for (int u = 0; u < 8; u++) {
                if (mu[u] == -INFINITY) continue;
                if (mu[u] > m) {
                    sum = (m == -INFINITY ? 0.0f : sum * __expf(m - mu[u])) + su[u];
                    m = mu[u];
                } else {
                    sum += su[u] * __expf(mu[u] - m);
                }
            }
        }
        for (; j0 < P; j0 += 32) {
            const int j = j0 + lane;
            visit(j, j < P ? l[j] : -INFINITY, j < P);
        }
        // warp-wide softmax normaliser
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float m2 = __shfl_xor_sync(0xffffffffu, m, o), s2 = __shfl_xor_sync(0xffffffffu, sum, o);
            const float mm = fmaxf(m, m2);
            sum = (m == -INFINITY ? 0.0f : sum * __expf(m - mm)) + (m2 == -INFINITY ? 0.0f : s2 * __expf(m2 - mm));
            m = mm;
        }
        if (cnt < min(h, P) || cnt > TK_CAP) {
            if (lane == 0) fail_rows[atomicAdd(fail_count, 1)] = (int)row;
            __syncwarp();
            continue;
        }
        __syncwarp();
        const int hh0 = min(h, P);
        int nk = cnt;
        if (cnt > 256 && hh0 <= 256) {
            // only the h largest keys are needed: the h-th largest by a radix
            // select over the kept (unique) keys, eight 8-bit digits from the
            // top, then the keys at or above it moved to the front, so that
            // the sort below covers 256 keys instead of 512 or 1,024
            unsigned long long pre = 0ull, msk = 0ull;
            int want = hh0;
            for (int pass = 0; pass < 8; pass++) {
                const int shift = 56 - 8 * pass;
                for (int i = lane; i < 256; i += 32) hist[i] = 0u;
                __syncwarp();
                for (int i = lane; i < cnt; i += 32) {
                    const unsigned long long k = buf[i];
                    if ((k & msk) == pre) atomicAdd(&hist[(unsigned)(k >> shift) & 255u], 1u);
                }
                __syncwarp();
                // digits from 255 down: lane l holds [248 - 8 l, 256 - 8 l)
                int mine = 0;
#pragma unroll
                for (int i = 0; i < 8; i++) mine += (int)hist[255 - (lane * 8 + i)];
                int incl = mine;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                const unsigned hit = __ballot_sync(0xffffffffu, incl >= want);
                const int L = __ffs(hit) - 1;
                int before = __shfl_sync(0xffffffffu, incl - mine, L);
                int digit = 0;
                if (lane == L) {
                    int c = before;
                    for (int i = 0; i < 8; i++) {
                        const int d = 255 - (L * 8 + i);
                        if (c + (int)hist[d] >= want) {
                            digit = d;
                            break;
                        }
                        c += (int)hist[d];
                    }
                    before = c;
                }
                digit = __shfl_sync(0xffffffffu, digit, L);
                before = __shfl_sync(0xffffffffu, before, L);
                want -= before;
                pre |= (unsigned long long)digit << shift;
                msk |= 255ull << shift;
                __syncwarp();
            }
            // pre is the h-th largest key: keep the keys >= it (exactly h),
            // compacted in place (a chunk is read before any lane writes)
            int out = 0;
            for (int i0 = 0; i0 < cnt; i0 += 32) {
                const int i = i0 + lane;
                const unsigned long long k = i < cnt ? buf[i] : 0ull;
                const bool keep = i < cnt && k >= pre;
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                __syncwarp();
                if (keep) buf[out + __popc(bal & ((1u << lane) - 1u))] = k;
                out += __popc(bal);
                __syncwarp();
            }
            nk = out;
        }
        int n2 = 1;
        while (n2 < nk) n2 <<= 1;
        for (int i = nk + lane; i < n2; i += 32) buf[i] = 0ull;
        __syncwarp();
        tk_warp_sort_desc(buf, n2);
        // the h largest, written ascending by (logit, index)
        const int hh = min(h, P);
        double part = 0.0;  // this lane's share of the candidate mass
        for (int i = lane; i < hh; i += 32) {
            const int j = (int)(buf[hh - 1 - i] & 0xffffffffu);
            const float pr = expf(l[j] - m) / sum;
            out_idx[row * h + i] = j;
            out_prob[row * h + i] = pr;
            part += (double)pr * (double)counts[j];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
        if (lane == 0) out_mass[row] = part;
        __syncwarp();
    }
}

// ------------------------------------------------------------------ launchers
cudaError_t wp_mlp_launch_input(const float* xf, const double* xd, int B, int TC, bf16* X, cudaStream_t s) {
    const long n = (long)B * 64;
    if (n == 0) return cudaSuccess;
    wp_mlp_input_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(xf, xd, B, TC, X);
    return cudaGetLastError();
}

cudaError_t wp_mlp_launch_transpose(const bf16* in, int rows, int cols, int ld_in, bf16* out, int ld_out,
                                    cudaStream_t s) {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
    wp_transpose_bf16_kernel<<<grid, block, 0, s>>>(in, rows, cols, ld_in, out, ld_out);
    return cudaGetLastError();
}

cudaError_t wp_mlp_launch_softmax_ce(const float* logits, int B, int P, int ld, const int* labels, float scale,
                                     bf16* dL, double* loss, cudaStream_t s) {
    wp_softmax_ce_kernel<<<B, 256, 0, s>>>(logits, P, ld, labels, scale, dL, loss);
    return cudaGetLastError();
}

cudaError_t wp_mlp_launch_gelu_bwd(const float* dH, const bf16* Z, long n, bf16* dZ, cudaStream_t s) {
    wp_gelu_bwd_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(dH, Z, n, dZ);
    return cudaGetLastError();
}

cudaError_t wp_mlp_launch_colsum(const bf16* M, int rows, int cols, int ld, float* out, cudaStream_t s) {
    wp_colsum_bf16_kernel<<<(cols + 255) / 256, 256, 0, s>>>(M, rows, cols, ld, out);
    return cudaGetLastError();
}

cudaError_t wp_mlp_launch_adam(float* w, const float* g, float* m, float* v, long n, float lr, float b1, float b2,
                               float eps, float bc1, float bc2, bf16* wb, cudaStream_t s) {
    wp_adam_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(w, g, m, v, n, lr, b1, b2, eps, bc1, bc2, wb);
    return cudaGetLastError();
}

cudaError_t wp_mlp_launch_to_bf16(const float* in, long n, bf16* out, cudaStream_t s) {
    wp_f32_to_bf16_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(in, n, out);
    return cudaGetLastError();
}

cudaError_t wp_mlp_launch_init(float* w, long rows, long cols, long valid_rows, float std, unsigned long long seed,
                               cudaStream_t s) {
    const long n = rows * cols;
    wp_init_normal_kernel<<<(int)((n + 255) / 256), 256, 0, s>>>(w, rows, cols, valid_rows, std, seed);
    return cudaGetLastError();
}

// fail: scratch of R + 1 ints (the fallback's row list, then its count).
cudaError_t wp_mlp_launch_topk(const float* logits, int R, int P, int ld, int h, const int* counts, int* idx,
                               float* prob, double* mass, int* fail, cudaStream_t s) {
    if (R == 0) return cudaSuccess;
    if (h > 1024) return cudaErrorInvalidValue;
    int* fail_count = fail + R;
    cudaError_t e = cudaMemsetAsync(fail_count, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    const size_t smem = sizeof(unsigned long long) * TK_WARPS * TK_CAP + sizeof(unsigned) * TK_WARPS * 256;
    int dev = 0;
    cudaGetDevice(&dev);
    // launch shape, once per device
    static int shape_sms[64] = {0}, shape_per_sm[64] = {0};
    static std::mutex shape_mu;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(shape_mu);
    if (shape_sms[dev] == 0) {
        e = cudaFuncSetAttribute(wp_topk_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        int sms0 = 0, per0 = 0;
        cudaDeviceGetAttribute(&sms0, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per0, wp_topk_warp_kernel, TK_WARPS * 32, smem);
        if (e != cudaSuccess) return e;
        shape_per_sm[dev] = per0;
        shape_sms[dev] = sms0;
    }
    const int sms = shape_sms[dev], per_sm = shape_per_sm[dev];
    const int grid = std::max(1, std::min(sms * std::max(per_sm, 1), (R + TK_WARPS - 1) / TK_WARPS));
    const int vec4 = (ld % 4 == 0 && ((uintptr_t)logits & 15u) == 0) ? 1 : 0;
    wp_topk_warp_kernel<<<grid, TK_WARPS * 32, smem, s>>>(logits, R, P, ld, h, counts, idx, prob, mass, fail,
                                                         fail_count, vec4);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // exact fallback for the reads the threshold missed (usually none)
    wp_topk_kernel<<<std::max(1, std::min(R, 2 * sms)), 256, 0, s>>>(logits, P, ld, h, counts, idx, prob, mass, fail,
                                                                       fail_count);
    return cudaGetLastError();
}

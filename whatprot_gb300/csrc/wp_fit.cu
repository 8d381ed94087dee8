// wp_fit.cu -- Baum-Welch E-step on the GPU: the expected counts of
// GenericHMM::improve_fit (hmm/hmm/generic-hmm.h:60-109) for every read of
// one dye-seq, summed in FP64.
//
// The reference fits without pruning (run-fit.cc:59 sets dist_cutoff to
// infinity) and with a single dye-seq, so every read has the same state
// shape: [Edman count e][dyes per channel] over the full extents D_c + 1.
// One thread runs one read; all threads of a warp follow the same control
// flow and their state vectors are interleaved in a global scratch slab
// (element k of thread i at k * nthreads + i), so every access is coalesced.
//
// Per read: a backward pass from the all-ones final vector stores the
// backward vector at each timestep boundary (a checkpoint, normalised by a
// power of two whose exponent is kept); a forward sweep then, timestep by
// timestep, recomputes the backward vectors between that timestep's steps
// from the next checkpoint, accumulates each step's expected counts
// (improve_fit of hmm/step/*.cc) and advances the forward vector, rescaled
// by a power of two after each emission.  Each term f * b / P is formed in
// FP32 from the scaled vectors and multiplied by the exact frame factor
// 2^(forward exponent + backward exponent - exponent of P) / P_mant, then
// added to per-thread FP64 sums; wp_fit_reduce_kernel adds the per-thread
// sums in a fixed order.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "wp_common.cuh"

// Sum slots per thread (doubles): the fitted rates' terms (FS_*, fs_*), then
// with the emission statistics 3 x C x WP_EMIS_N more (fs_emis).
#define WP_EMIS_N (WP_MAX_DYES_PER_CHANNEL + 1)
__host__ __device__ inline int fit_nslots_rates(int T, int C) { return 6 + 2 * (T - 1) + 4 * C; }
__host__ __device__ inline int fit_nslots(int T, int C, bool emission) {
    return fit_nslots_rates(T, C) + (emission ? 3 * C * WP_EMIS_N : 0);
}
// kind 0: posterior weight, 1: weight x intensity, 2: weight x intensity^2
__host__ __device__ inline int fs_emis(int T, int C, int kind, int c, int n) {
    return fit_nslots_rates(T, C) + (kind * C + c) * WP_EMIS_N + n;
}
#define FS_EDMAN_NUM 0
#define FS_EDMAN_DEN 1
#define FS_IB_NUM 2
#define FS_IB_DEN 3
#define FS_CB_NUM 4
#define FS_CB_DEN 5
__host__ __device__ inline int fs_det_x(int t) { return 6 + 2 * t; }
__host__ __device__ inline int fs_det_n(int t) { return 7 + 2 * t; }
__host__ __device__ inline int fs_bleach_num(int T, int c) { return 6 + 2 * (T - 1) + 4 * c; }
__host__ __device__ inline int fs_bleach_den(int T, int c) { return 7 + 2 * (T - 1) + 4 * c; }
__host__ __device__ inline int fs_dud_num(int T, int c) { return 8 + 2 * (T - 1) + 4 * c; }
__host__ __device__ inline int fs_dud_den(int T, int c) { return 9 + 2 * (T - 1) + 4 * c; }



// A state vector of thread `tid`: A and B tensors of up to T*S states (B
// only with blocking) and the detached-state scalar.  Element k of A lives
// at base[k * nt], of B at base[(cap + k) * nt], pd after them.
struct Vec {
    float* base;
    long nt;
    long cap;
    long pd_at;  // cap (no blocking) or 2 * cap
    __device__ float& A(long k) const { return base[k * nt]; }
    __device__ float& B(long k) const { return base[(cap + k) * nt]; }
    __device__ float& pd() const { return base[pd_at * nt]; }
};

template <bool HB>
__device__ void vec_fill(const Vec& v, long n, float val) {
    for (long k = 0; k < n; k++) {
        v.A(k) = val;
        if (HB) v.B(k) = val;
    }
    v.pd() = val;
}

// Multiply a vector of n states by 2^-k (exact).
template <bool HB>
__device__ void vec_scale_pow2(const Vec& v, long n, int k) {
    const float f = exp2i(-k);
    for (long i = 0; i < n; i++) {
        v.A(i) *= f;
        if (HB) v.B(i) *= f;
    }
    v.pd() *= f;
}

struct Shape {
    int C, S;
    int W[WP_MAX_CHANNELS];   // D_c + 1
    int st[WP_MAX_CHANNELS];  // strides of the dye-count index
};

__device__ inline int coord(const Shape& sh, int j, int c) { return (j / sh.st[c]) % sh.W[c]; }

// Emission factor of dye-count index j at timestep t, normalised by 2^kmax.
__device__ inline float emit_at(const FitArgs& a, const EmitEntry* tab, const Shape& sh, int t, int j, int kmax) {
    float mm = 1.0f;
    int ks = 0;
    for (int c = 0; c < sh.C; c++) {
        EmitEntry en = tab[(t * sh.C + c) * a.W + coord(sh, j, c)];
        mm *= en.mant;
        ks += en.expo;
    }
    return mm != 0.0f ? mm * exp2i(max(ks - kmax, -200)) : 0.0f;
}

__device__ inline int emit_kmax(const FitArgs& a, const EmitEntry* tab, const Shape& sh, int t) {
    int kmax = 0;
    for (int c = 0; c < sh.C; c++) {
        int km = WP_EXPO_ZERO;
        for (int n = 0; n < sh.W[c]; n++) {
            EmitEntry en = tab[(t * sh.C + c) * a.W + n];
            if (en.mant != 0.0f) km = max(km, en.expo);
        }
        if (km == WP_EXPO_ZERO) return WP_EXPO_ZERO;
        kmax += km;
    }
    return kmax;
}

// out = binomial transition of `in` along channel c over E slices
// (forward, binomial-transition.cc:114-136) or its transpose (backward,
// :161-183).  Full extents.
template <bool HB>
__device__ void binomial_full(const Vec& in, const Vec& out, const Shape& sh, int E, int c,
                              const float* tab, bool backward) {
    const int Wc = sh.W[c], stc = sh.st[c];
    const int F = sh.S / Wc;
    for (int e = 0; e < E; e++) {
        for (int f = 0; f < F; f++) {
            // fiber base: index with n_c = 0
            int rem = f, j0 = 0;
            for (int c2 = sh.C - 1; c2 >= 0; c2--) {
                if (c2 == c) continue;
                j0 += (rem % sh.W[c2]) * sh.st[c2];
                rem /= sh.W[c2];
            }
            const long b = (long)e * sh.S + j0;
            for (int x = 0; x < Wc; x++) {
                float acc = 0.0f, accb = 0.0f;
                if (!backward) {  // out[to = x] = sum_{from >= x} prob(from, x) in[from]
                    for (int from = x; from < Wc; from++) {
                        const float p = tab[from * (from + 1) / 2 + x];
                        acc = fmaf(p, in.A(b + from * stc), acc);
                        if (HB) accb = fmaf(p, in.B(b + from * stc), accb);
                    }
                } else {  // out[from = x] = sum_{to <= x} prob(x, to) in[to]
                    for (int to = 0; to <= x; to++) {
                        const float p = tab[x * (x + 1) / 2 + to];
                        acc = fmaf(p, in.A(b + to * stc), acc);
                        if (HB) accb = fmaf(p, in.B(b + to * stc), accb);
                    }
                }
                out.A(b + x * stc) = acc;
                if (HB) out.B(b + x * stc) = accb;
            }
        }
    }
    out.pd() = in.pd();
}

// Expected counts of a binomial step (binomial-transition.cc:232-256):
// den += sum_{from >= 1} f b / P * from, num += sum_{to < from} f prob nb / P * (from - to).
template <bool HB>
__device__ void binomial_em(const Vec& f, const Vec& b, const Vec& nb, const Shape& sh, int E, int c,
                            const float* tab, double scale, double* num, double* den) {
    const int Wc = sh.W[c], stc = sh.st[c];
    const int F = sh.S / Wc;
    float n32 = 0.0f, d32 = 0.0f;
    for (int e = 0; e < E; e++) {
        for (int fi = 0; fi < F; fi++) {
            int rem = fi, j0 = 0;
            for (int c2 = sh.C - 1; c2 >= 0; c2--) {
                if (c2 == c) continue;
                j0 += (rem % sh.W[c2]) * sh.st[c2];
                rem /= sh.W[c2];
            }
            const long base = (long)e * sh.S + j0;
            for (int from = 1; from < Wc; from++) {
                const float fa = f.A(base + from * stc);
                d32 = fmaf(fa * b.A(base + from * stc), (float)from, d32);
                for (int to = 0; to < from; to++)
                    n32 = fmaf(fa * tab[from * (from + 1) / 2 + to] * nb.A(base + to * stc), (float)(from - to), n32);
                if (HB) {
                    const float fb = f.B(base + from * stc);
                    d32 = fmaf(fb * b.B(base + from * stc), (float)from, d32);
                    for (int to = 0; to < from; to++)
                        n32 = fmaf(fb * tab[from * (from + 1) / 2 + to] * nb.B(base + to * stc), (float)(from - to), n32);
                }
            }
        }
    }
    *num += (double)n32 * scale;
    *den += (double)d32 * scale;
}

// One E-step for one read.  Returns log P (−inf when P == 0: no counts).
template <bool HB>
__device__ double fit_read(const FitArgs& a, const SmemModel& M, int r, const Shape& sh, float* base, long nt,
                           double* sums) {
    const DevModel& m = *a.model;
    const int T = m.T, C = sh.C, S = sh.S;
    const long cap = (long)T * S;
    const long vstride = (HB ? 2 : 1) * cap + 1;  // floats per vector
    const EmitEntry* tab = a.tab + (long)r * T * C * a.W;
    // Vector slots: checkpoints 1..T-1 (cp[t] has t slices), the T
    // boundary vectors of one timestep (C + 5), two forward vectors.
    auto vec = [&](int slot) {
        Vec v;
        v.base = base + (long)slot * vstride * nt;
        v.nt = nt;
        v.cap = cap;
        v.pd_at = (HB ? 2 : 1) * cap;
        return v;
    };
    const int CP0 = 0;              // checkpoint t at slot CP0 + t (t = 0..T)
    const int BW0 = T + 1;          // boundary vectors b0..b_{C+4}
    const int AL0 = BW0 + C + 5;    // forward vectors (2)
    int kmx[WP_MAX_TIMESTEPS];
    for (int t = 0; t < T; t++) kmx[t] = emit_kmax(a, tab, sh, t);
    for (int t = 0; t < T; t++)
        if (kmx[t] == WP_EXPO_ZERO) return -INFINITY;  // some timestep emits nothing
    const float pf = m.pf, qf = 1.0f - m.pf;

    // Backward through timestep t's chain from vector `out_v` (= cp t+1)
    // into the boundary vectors; fills b[0..C+4] (b[C+4] = out_v copy).
    // Step order: b0 in(CB) -> b1 in(DT) -> b2+c in(BL c) -> b2+C in(ED) ->
    // b3+C in(EM) -> b4+C out(EM).
    auto backward_timestep = [&](int t, const Vec& out_v, Vec* bv) {
        const int kmax = kmx[t];
        // emission (forward_or_backward, peptide-emission.cc:212-243); the
        // unpruned box always includes zero, so allow_detached holds.
        const long n1 = (long)(t + 1) * S;
        for (long i = 0; i < n1; i++) {
            const float w = emit_at(a, tab, sh, t, (int)(i % S), kmax);
            bv[3 + C].A(i) = w * out_v.A(i);
            if (HB) bv[3 + C].B(i) = w * out_v.B(i);
        }
        bv[3 + C].pd() = emit_at(a, tab, sh, t, 0, kmax) * out_v.pd();
        // Edman transpose (edman-transition.cc:164-277) as a gather.
        const long n0 = (long)t * S;
        for (int e = 0; e < t; e++) {
            const int dc = a.dye[e];
            const float tot = dc >= 0 ? (float)a.tot[e] : 1.0f;
            for (int j = 0; j < S; j++) {
                const long i = (long)e * S + j;
                float v = pf * bv[3 + C].A(i);
                if (dc < 0) {
                    v = fmaf(qf, bv[3 + C].A(i + S), v);
                } else {
                    const int nc = coord(sh, j, dc);
                    if ((float)nc < tot) v = fmaf(qf * (1.0f - (float)nc / tot), bv[3 + C].A(i + S), v);
                    if (nc >= 1) v = fmaf(qf * ((float)nc / tot), bv[3 + C].A(i + S - sh.st[dc]), v);
                }
                bv[2 + C].A(i) = v;
                if (HB) bv[2 + C].B(i) = bv[3 + C].B(i);
            }
        }
        bv[2 + C].pd() = bv[3 + C].pd();
        // bleach transposes, channel C-1 .. 0
        for (int c = C - 1; c >= 0; c--) binomial_full<HB>(bv[3 + c], bv[2 + c], sh, t, c, M.bleach[c], true);
        // detach transpose (detach-transition.cc:70-103)
        const float pdt = M.p_det[t - 1];
        for (long i = 0; i < n0; i++) {
            bv[1].A(i) = fmaf(1.0f - pdt, bv[2].A(i), pdt * bv[2].pd());
            if (HB) bv[1].B(i) = fmaf(1.0f - pdt, bv[2].B(i), pdt * bv[2].pd());
        }
        bv[1].pd() = bv[2].pd();
        // cyclic block transpose (block-transition.cc:64-93)
        for (long i = 0; i < n0; i++) {
            if (HB) {
                bv[0].A(i) = fmaf(m.p_cb, bv[1].B(i), (1.0f - m.p_cb) * bv[1].A(i));
                bv[0].B(i) = bv[1].B(i);
            } else {
                bv[0].A(i) = (1.0f - m.p_cb) * bv[1].A(i);
            }
        }
        bv[0].pd() = bv[1].pd();
    };
    // Same for the t = 0 chain: d0 in(IB) -> d1+c in(DD c) -> d1+C in(EM0) -> out.
    auto backward_t0 = [&](const Vec& out_v, Vec* bv) {
        const int kmax = kmx[0];
        for (int j = 0; j < S; j++) {
            const float w = emit_at(a, tab, sh, 0, j, kmax);
            bv[1 + C].A(j) = w * out_v.A(j);
            if (HB) bv[1 + C].B(j) = w * out_v.B(j);
        }
        bv[1 + C].pd() = emit_at(a, tab, sh, 0, 0, kmax) * out_v.pd();
        for (int c = C - 1; c >= 0; c--) binomial_full<HB>(bv[2 + c], bv[1 + c], sh, 1, c, M.dud[c], true);
        for (int j = 0; j < S; j++) {
            if (HB) {
                bv[0].A(j) = fmaf(m.p_ib, bv[1].B(j), (1.0f - m.p_ib) * bv[1].A(j));
                bv[0].B(j) = bv[1].B(j);
            } else {
                bv[0].A(j) = (1.0f - m.p_ib) * bv[1].A(j);
            }
        }
        bv[0].pd() = bv[1].pd();
    };
    Vec bv[WP_MAX_CHANNELS + 5];
    for (int k = 0; k < C + 5; k++) bv[k] = vec(BW0 + k);

    // ---- backward pass: checkpoints cp[t] = backward vector at the input of
    // timestep t's chain, with exponents Eb[t] (true = stored * 2^Eb).
    int Eb[WP_MAX_TIMESTEPS + 1];
    {
        Vec last = vec(CP0 + T);
        vec_fill<HB>(last, (long)T * S, 1.0f);  // initialize_from_finish
        Eb[T] = 0;
        for (int t = T - 1; t >= 1; t--) {
            backward_timestep(t, vec(CP0 + t + 1), bv);
            // normalise by the exponent of the largest entry
            float mx = bv[0].pd();
            const long n0 = (long)t * S;
            for (long i = 0; i < n0; i++) {
                mx = fmaxf(mx, bv[0].A(i));
                if (HB) mx = fmaxf(mx, bv[0].B(i));
            }
            int k = 0;
            if (mx > 0.0f) frexpf(mx, &k);
            Vec cp = vec(CP0 + t);
            for (long i = 0; i < n0; i++) {
                cp.A(i) = bv[0].A(i);
                if (HB) cp.B(i) = bv[0].B(i);
            }
            cp.pd() = bv[0].pd();
            vec_scale_pow2<HB>(cp, n0, k);
            Eb[t] = Eb[t + 1] + kmx[t] + k;
        }
        if (T == 1) {
            // the chain ends at emission 0: backward from the all-ones vector
        }
        backward_t0(vec(CP0 + 1), bv);
        Eb[0] = Eb[1] + kmx[0];
    }
    // P = source of the backward vector (peptide-state-vector.cc:56-58):
    // the start state (0, D) is the last index of slice 0.
    const float Ps = bv[0].A(S - 1);
    if (!(Ps > 0.0f)) return -INFINITY;  // improve_fit returns early (generic-hmm.h:85-87)
    int EP;
    const float Pm = frexpf(Ps, &EP);
    EP += Eb[0];
    const double logP = log((double)Pm) + (double)EP * 0.69314718055994530942;
    // scale(t) = 2^(Ea + Eb_chain - EP) / Pm, the factor turning f*b products of
    // the scaled vectors into f*b/P.
    auto scale_of = [&](int Ea, int Ebc) { return ldexp(1.0 / (double)Pm, Ea + Ebc - EP); };

    // Emission statistics at emission t (no reference counterpart): the
    // posterior f * b / P of each state (f the forward vector before the
    // emission, b the backward vector at its input), binned by each
    // channel's dye count; the detached state shows 0 on every channel.
    auto emis_gather = [&](int t, const Vec& f, const Vec& b, long n1, double sc) {
        const double* x = a.rads + ((long)r * T + t) * C;
        for (long i = 0; i < n1; i++) {
            float g = f.A(i) * b.A(i);
            if (HB) g = fmaf(f.B(i), b.B(i), g);
            if (g == 0.0f) continue;
            const double gs = (double)g * sc;
            const int j = (int)(i % S);
            for (int c = 0; c < C; c++) {
                const int n = coord(sh, j, c);
                sums[fs_emis(T, C, 0, c, n) * nt] += gs;
                sums[fs_emis(T, C, 1, c, n) * nt] += gs * x[c];
                sums[fs_emis(T, C, 2, c, n) * nt] += gs * x[c] * x[c];
            }
        }
        const double gd = (double)(f.pd() * b.pd()) * sc;
        for (int c = 0; c < C; c++) {
            sums[fs_emis(T, C, 0, c, 0) * nt] += gd;
            sums[fs_emis(T, C, 1, c, 0) * nt] += gd * x[c];
            sums[fs_emis(T, C, 2, c, 0) * nt] += gd * x[c] * x[c];
        }
    };

    // ---- forward sweep with the expected counts.
    Vec al = vec(AL0), an = vec(AL0 + 1);
    // t = 0 chain: initial block, duds, emission 0.
    vec_fill<HB>(al, S, 0.0f);
    al.A(S - 1) = 1.0f;  // initialize_from_start
    int Ea = 0;
    {
        backward_t0(vec(CP0 + 1), bv);  // d0..d_{1+C} in frame Eb[1] + kmx[0] ... (Eb[0])
        const double sc = scale_of(Ea, Eb[0]);
        // initial block EM (block-transition.cc:95-116): num += f p nb.B, den += f b
        {
            float n32 = 0.0f, d32 = 0.0f;
            for (int j = 0; j < S; j++) {
                const float f = al.A(j);
                if (HB) n32 = fmaf(f * m.p_ib, bv[1].B(j), n32);
                d32 = fmaf(f, bv[0].A(j), d32);
            }
            sums[FS_IB_NUM * nt] += (double)n32 * sc;
            sums[FS_IB_DEN * nt] += (double)d32 * sc;
        }
        if (HB) {
            for (int j = 0; j < S; j++) {
                const float f = al.A(j);
                al.B(j) = al.B(j) + m.p_ib * f;
                al.A(j) = (1.0f - m.p_ib) * f;
            }
        } else {
            for (int j = 0; j < S; j++) al.A(j) = (1.0f - m.p_ib) * al.A(j);
        }
        for (int c = 0; c < C; c++) {
            binomial_em<HB>(al, bv[1 + c], bv[2 + c], sh, 1, c, M.dud[c], sc, &sums[fs_dud_num(T, c) * nt],
                            &sums[fs_dud_den(T, c) * nt]);
            binomial_full<HB>(al, an, sh, 1, c, M.dud[c], false);
            Vec tmp = al;
            al = an;
            an = tmp;
        }
        if (a.emission) emis_gather(0, al, bv[1 + C], S, sc);
        // emission 0 and rescale
        const int kmax = kmx[0];
        float tot = 0.0f;
        for (int j = 0; j < S; j++) {
            const float w = emit_at(a, tab, sh, 0, j, kmax);
            al.A(j) *= w;
            tot += al.A(j);
            if (HB) {
                al.B(j) *= w;
                tot += al.B(j);
            }
        }
        al.pd() *= emit_at(a, tab, sh, 0, 0, kmax);
        tot += al.pd();
        Ea += kmax;
        int k = 0;
        if (tot > 0.0f) frexpf(tot, &k);
        vec_scale_pow2<HB>(al, S, k);
        Ea += k;
    }
    for (int t = 1; t < T; t++) {
        // backward vectors of this timestep, frame Eb[t+1] + kmx[t] after the
        // emission transpose: every b here shares the frame of cp[t+1] times
        // 2^kmx[t] (the emission factors are normalised by 2^-kmx[t]).
        backward_timestep(t, vec(CP0 + t + 1), bv);
        const double sc = scale_of(Ea, Eb[t + 1] + kmx[t]);
        const long n0 = (long)t * S;
        // cyclic block EM
        {
            float n32 = 0.0f, d32 = 0.0f;
            for (long i = 0; i < n0; i++) {
                const float f = al.A(i);
                if (HB) n32 = fmaf(f * m.p_cb, bv[1].B(i), n32);
                d32 = fmaf(f, bv[0].A(i), d32);
            }
            sums[FS_CB_NUM * nt] += (double)n32 * sc;
            sums[FS_CB_DEN * nt] += (double)d32 * sc;
        }
        if (HB) {
            for (long i = 0; i < n0; i++) {
                const float f = al.A(i);
                al.B(i) = al.B(i) + m.p_cb * f;
                al.A(i) = (1.0f - m.p_cb) * f;
            }
        } else {
            for (long i = 0; i < n0; i++) al.A(i) = (1.0f - m.p_cb) * al.A(i);
        }
        // detach EM (detach-transition.cc:121-166), skipping the all-zero
        // dye-count state of each Edman slice; then the transition.
        {
            const float pdt = M.p_det[t - 1];
            float fs = 0.0f, fb = 0.0f, all = 0.0f;
            for (int e = 0; e < t; e++)
                for (int j = 0; j < S; j++) {
                    const long i = (long)e * S + j;
                    const float f = al.A(i);
                    all += f;
                    if (j != 0) {
                        fs += f;
                        fb = fmaf(f, bv[1].A(i), fb);
                    }
                    if (HB) {
                        const float g = al.B(i);
                        all += g;
                        if (j != 0) {
                            fs += g;
                            fb = fmaf(g, bv[1].B(i), fb);
                        }
                    }
                }
            sums[fs_det_x(t - 1) * nt] += (double)(fs * pdt) * (double)bv[2].pd() * sc;
            sums[fs_det_n(t - 1) * nt] += (double)fb * sc;
            for (long i = 0; i < n0; i++) {
                al.A(i) *= 1.0f - pdt;
                if (HB) al.B(i) *= 1.0f - pdt;
            }
            al.pd() = al.pd() + pdt * all;
        }
        // bleach per channel
        for (int c = 0; c < C; c++) {
            binomial_em<HB>(al, bv[2 + c], bv[3 + c], sh, t, c, M.bleach[c], sc, &sums[fs_bleach_num(T, c) * nt],
                            &sums[fs_bleach_den(T, c) * nt]);
            binomial_full<HB>(al, an, sh, t, c, M.bleach[c], false);
            Vec tmp = al;
            al = an;
            an = tmp;
        }
        // Edman EM (edman-transition.cc:279-325) over e < t, skipping the
        // all-zero state of each slice; then the transition (gather form).
        {
            float n32 = 0.0f, d32 = 0.0f;
            for (int e = 0; e < t; e++)
                for (int j = 1; j < S; j++) {
                    const long i = (long)e * S + j;
                    const float f = al.A(i);
                    n32 = fmaf(f * pf, bv[3 + C].A(i), n32);
                    d32 = fmaf(f, bv[2 + C].A(i), d32);
                }
            sums[FS_EDMAN_NUM * nt] += (double)n32 * sc;
            sums[FS_EDMAN_DEN * nt] += (double)d32 * sc;
            for (int e = 0; e <= t; e++) {
                const int dc = e >= 1 ? a.dye[e - 1] : -1;
                const float tot = dc >= 0 ? (float)a.tot[e - 1] : 1.0f;
                for (int j = 0; j < S; j++) {
                    const long i = (long)e * S + j;
                    float v = e < t ? pf * al.A(i) : 0.0f;
                    if (e >= 1) {
                        const float xin = al.A(i - S);
                        if (dc < 0) {
                            v = fmaf(qf, xin, v);
                        } else {
                            const int nc = coord(sh, j, dc);
                            if ((float)nc < tot) v = fmaf(qf * (1.0f - (float)nc / tot), xin, v);
                            if (nc + 1 < sh.W[dc])
                                v = fmaf(qf * ((float)(nc + 1) / tot), al.A(i - S + sh.st[dc]), v);
                        }
                    }
                    an.A(i) = v;
                    if (HB) an.B(i) = e < t ? al.B(i) : 0.0f;
                }
            }
            an.pd() = al.pd();
            Vec tmp = al;
            al = an;
            an = tmp;
        }
        if (a.emission) emis_gather(t, al, bv[3 + C], (long)(t + 1) * S, sc);
        // emission t and rescale
        {
            const int kmax = kmx[t];
            const long n1 = (long)(t + 1) * S;
            float tot = 0.0f;
            for (long i = 0; i < n1; i++) {
                const float w = emit_at(a, tab, sh, t, (int)(i % S), kmax);
                al.A(i) *= w;
                tot += al.A(i);
                if (HB) {
                    al.B(i) *= w;
                    tot += al.B(i);
                }
            }
            al.pd() *= emit_at(a, tab, sh, t, 0, kmax);
            tot += al.pd();
            Ea += kmax;
            int k = 0;
            if (tot > 0.0f) frexpf(tot, &k);
            vec_scale_pow2<HB>(al, n1, k);
            Ea += k;
        }
    }
    return logP;
}

template <bool HB>
__global__ void __launch_bounds__(128) wp_fit_estep_kernel(FitArgs a) {
    __shared__ SmemModel M;
    load_smem_model(M, *a.model);
    __syncthreads();
    const long nt = (long)gridDim.x * blockDim.x;
    const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    Shape sh;
    sh.C = a.model->C;
    sh.S = 1;
    for (int c = sh.C - 1; c >= 0; c--) {
        sh.W[c] = a.D[c] + 1;
        sh.st[c] = sh.S;
        sh.S *= sh.W[c];
    }
    float* base = a.scratch + tid;
    double* sums = a.sums + tid;
    for (int k = 0; k < a.nslots; k++) sums[k * nt] = 0.0;
    for (long r = tid; r < a.R; r += nt) {
        double lp = fit_read<HB>(a, M, (int)r, sh, base, nt, sums);
        if (a.logp) a.logp[r] = lp;
    }
}

// Deterministic sum over threads: one thread per slot, fixed order.
__global__ void wp_fit_reduce_kernel(const double* __restrict__ sums, long nthreads, int nslots,
                                     double* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nslots) return;
    double s = 0.0;
    for (long i = 0; i < nthreads; i++) s += sums[(long)k * nthreads + i];
    out[k] = s;
}

int wp_fit_nslots(int T, int C, bool emission) { return fit_nslots(T, C, emission); }

// Floats of scratch per thread: (T + 1) checkpoints, C + 5 boundary
// vectors and 2 forward vectors, each (1 or 2) * T * S + 1 floats.
long wp_fit_floats_per_thread(int T, int C, int S, bool has_block) {
    return (long)(T + 1 + C + 5 + 2) * ((has_block ? 2L : 1L) * T * S + 1);
}

cudaError_t wp_launch_fit_estep(bool has_block, int grid, int threads, cudaStream_t s, const FitArgs& a) {
    if (has_block)
        wp_fit_estep_kernel<true><<<grid, threads, 0, s>>>(a);
    else
        wp_fit_estep_kernel<false><<<grid, threads, 0, s>>>(a);
    return cudaGetLastError();
}

// ===========================================================================
// CTA-per-read E-step.  The same computation as wp_fit_estep_kernel, with
// one read per CTA at a time (persistent over reads) and the states spread
// over the CTA's threads: the backward vectors of one timestep, the current
// backward vector and two forward vectors live in shared memory; only the
// T+1 checkpoints go to global memory (per-CTA slots, L2-resident for a
// persistent grid).  Per-term FP32 partials are reduced across the CTA once
// per timestep in a fixed order and accumulated in FP64 per CTA; the CTAs'
// sums are added in CTA order by wp_fit_reduce_kernel.
// ===========================================================================
#define FIT_NT 256
#define FIT_MAXTERMS (6 + 2 * WP_MAX_CHANNELS)
#define FIT_EMIS_BUCKETS (WP_MAX_CHANNELS * WP_EMIS_N)

// Loop over state indices i = tid, tid + NT, ... < n with the slice e = i / S
// and dye-count index j = i % S kept incrementally (no division per state).
#define FOR_STATES(n, S, i, e, j)                                                                  \
    for (long i = threadIdx.x, e = threadIdx.x / (S), j = threadIdx.x % (S); i < (n);              \
         i += blockDim.x, e += blockDim.x / (S), j += blockDim.x % (S), e += (j >= (S)) ? 1 : 0, \
              j -= (j >= (S)) ? (S) : 0)

struct SVec {
    float* A;
    float* B;
    float* pd;
};

__device__ __forceinline__ int fcoord(const uint32_t* coords, int j, int c) { return (coords[j] >> (4 * c)) & 15; }

// Sum (or max) of n values per thread across the CTA, fixed order: shuffle
// tree per warp, then warp 0 over the warps.  Result in out[0..n) for all.
template <bool MAX>
__device__ void cta_reduce(float* v, int n, float* red, float* out) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < n; k++) {
        float x = v[k];
        for (int o = 16; o > 0; o >>= 1) {
            const float y = __shfl_down_sync(0xffffffffu, x, o);
            x = MAX ? fmaxf(x, y) : x + y;
        }
        if (lane == 0) red[k * 32 + w] = x;
    }
    __syncthreads();
    if (w == 0) {
        for (int k = 0; k < n; k++) {
            float x = lane < nw ? red[k * 32 + lane] : (MAX ? -INFINITY : 0.f);
            for (int o = 16; o > 0; o >>= 1) {
                const float y = __shfl_down_sync(0xffffffffu, x, o);
                x = MAX ? fmaxf(x, y) : x + y;
            }
            if (lane == 0) out[k] = x;
        }
    }
    __syncthreads();
}

// Emission statistics of one emission (no reference counterpart): g = f * b
// per state (f the forward vector before the emission, b the backward vector
// at its input) into the scratch g, then warp w sums buckets w, w + nw, ...
// (bucket k = channel c, dye count n, channels in order) over the states in
// a fixed order into ebk[k].
template <bool HB>
__device__ void cta_emission_buckets(const SVec& f, const SVec& b, float* g, long n1, int S, int C, const int* W,
                                     const uint32_t* coords, float* ebk) {
    for (long i = threadIdx.x; i < n1; i += blockDim.x) {
        float v = f.A[i] * b.A[i];
        if (HB) v = fmaf(f.B[i], b.B[i], v);
        g[i] = v;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int nb = 0;
    for (int c = 0; c < C; c++) nb += W[c];
    for (int k = w; k < nb; k += nw) {
        int c = 0, n = k;
        while (n >= W[c]) {
            n -= W[c];
            c++;
        }
        float sum = 0.0f;
        for (int j = lane; j < S; j += 32)
            if (fcoord(coords, j, c) == n)
                for (long i = j; i < n1; i += S) sum += g[i];
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
        if (lane == 0) ebk[k] = sum;
    }
    __syncthreads();
}

template <bool HB>
__device__ __forceinline__ void cta_emit(const SVec& in, const SVec& out, const float* w, int S, long n) {
    FOR_STATES(n, S, i, e, j) {
        const float f = w[j];
        out.A[i] = f * in.A[i];
        if (HB) out.B[i] = f * in.B[i];
    }
    if (threadIdx.x == 0) *out.pd = w[0] * *in.pd;
    __syncthreads();
}

// Binomial along channel c over E slices: forward (out[x] = sum_{from >= x}
// p(from, x) in[from]) or its transpose.
template <bool HB>
__device__ void cta_binomial(const SVec& in, const SVec& out, const uint32_t* coords, int S, int E, int c, int Wc,
                             int stc, const float* tab, bool backward) {
    const long n = (long)E * S;
    FOR_STATES(n, S, i, e, j) {
        const int x = fcoord(coords, (int)j, c);
        float acc = 0.f, accb = 0.f;
        if (!backward) {
            for (int from = x; from < Wc; from++) {
                const float p = tab[from * (from + 1) / 2 + x];
                const long k = i + (long)(from - x) * stc;
                acc = fmaf(p, in.A[k], acc);
                if (HB) accb = fmaf(p, in.B[k], accb);
            }
        } else {
            for (int to = 0; to <= x; to++) {
                const float p = tab[x * (x + 1) / 2 + to];
                const long k = i - (long)(x - to) * stc;
                acc = fmaf(p, in.A[k], acc);
                if (HB) accb = fmaf(p, in.B[k], accb);
            }
        }
        out.A[i] = acc;
        if (HB) out.B[i] = accb;
    }
    if (threadIdx.x == 0) *out.pd = *in.pd;
    __syncthreads();
}

template <bool HB>
__global__ void __launch_bounds__(FIT_NT) wp_fit_cta_kernel(FitArgs a, float* ckpt, long ck_stride) {
    __shared__ SmemModel M;
    extern __shared__ __align__(16) unsigned char fit_smem[];
    // batched instances: this CTA's instance and its place among the
    // instance's CTAs
    const int inst = a.inst_ctas > 0 ? (int)(blockIdx.x / a.inst_ctas) : 0;
    const long lb = a.inst_ctas > 0 ? (long)(blockIdx.x % a.inst_ctas) : (long)blockIdx.x;
    const long gs = a.inst_ctas > 0 ? (long)a.inst_ctas : (long)gridDim.x;
    const DevModel& m = a.model[inst];
    const int T = m.T, C = m.C;
    int W[WP_MAX_CHANNELS], st[WP_MAX_CHANNELS];
    int S = 1;
    for (int c = C - 1; c >= 0; c--) {
        W[c] = a.D[c] + 1;
        st[c] = S;
        S *= W[c];
    }
    const long cap = (long)T * S;
    const long VS = (((HB ? 2 : 1) * cap + 1) + 3) / 4 * 4;
    const int NV = C + 8;
    float* vbase = reinterpret_cast<float*>(fit_smem);
    float* wemit = vbase + NV * VS;                     // [T][S]
    uint32_t* coords = reinterpret_cast<uint32_t*>(wemit + (long)T * S);  // [S]
    float* red = reinterpret_cast<float*>(coords + S);  // [FIT_MAXTERMS][32]
    float* rout = red + FIT_MAXTERMS * 32;              // [FIT_MAXTERMS]
    float* ebk = rout + FIT_MAXTERMS;                    // [FIT_EMIS_BUCKETS]
    int* kmx = reinterpret_cast<int*>(ebk + FIT_EMIS_BUCKETS);  // [T]
    int* Eb = kmx + WP_MAX_TIMESTEPS;                   // [T + 1]
    double* acc = reinterpret_cast<double*>(((reinterpret_cast<uintptr_t>(Eb + WP_MAX_TIMESTEPS + 2)) + 7) & ~(uintptr_t)7);
    auto vec = [&](int slot) {
        SVec v;
        v.A = vbase + (long)slot * VS;
        v.B = v.A + cap;
        v.pd = v.A + (HB ? 2 : 1) * cap;
        return v;
    };
    auto gvec = [&](int t) {  // checkpoint t of this CTA (global)
        SVec v;
        v.A = ckpt + (long)blockIdx.x * ck_stride + (long)t * VS;
        v.B = v.A + cap;
        v.pd = v.A + (HB ? 2 : 1) * cap;
        return v;
    };
    load_smem_model(M, m);
    for (int j = threadIdx.x; j < S; j += blockDim.x) {
        uint32_t pk = 0;
        for (int c = 0; c < C; c++) pk |= (uint32_t)((j / st[c]) % W[c]) << (4 * c);
        coords[j] = pk;
    }
    for (int k = threadIdx.x; k < a.nslots; k += blockDim.x) acc[k] = 0.0;
    __syncthreads();
    const float pf = m.pf, qf = 1.0f - m.pf;
    const int BV = 0, CUR = C + 5, F0 = C + 6, F1 = C + 7;

    for (long kr = lb; kr < a.R; kr += gs) {
        const long r = a.read_idx ? (long)a.read_idx[(long)inst * a.R + kr] : kr;  // the read
        const long ro = a.read_idx ? (long)inst * a.R + kr : kr;                    // its output slot
        const EmitEntry* tab = a.tab + r * (long)T * C * a.W;
        // ---- emission weights per (t, j), normalised by 2^kmax[t]
        for (int t = threadIdx.x; t < T; t += blockDim.x) {
            int kmax = 0;
            for (int c = 0; c < C; c++) {
                int km = WP_EXPO_ZERO;
                for (int n = 0; n < W[c]; n++) {
                    const EmitEntry en = tab[(t * C + c) * a.W + n];
                    if (en.mant != 0.0f) km = max(km, en.expo);
                }
                if (km == WP_EXPO_ZERO) {
                    kmax = WP_EXPO_ZERO;
                    break;
                }
                kmax += km;
            }
            kmx[t] = kmax;
        }
        __syncthreads();
        bool dead = false;
        for (int t = 0; t < T; t++)
            if (kmx[t] == WP_EXPO_ZERO) dead = true;
        if (dead) {  // some timestep emits nothing: P = 0
            if (threadIdx.x == 0 && a.logp) a.logp[ro] = -INFINITY;
            __syncthreads();
            continue;
        }
        for (long i = threadIdx.x; i < (long)T * S; i += blockDim.x) {
            const int t = (int)(i / S), j = (int)(i % S);
            float mm = 1.0f;
            int ks = 0;
            for (int c = 0; c < C; c++) {
                const EmitEntry en = tab[(t * C + c) * a.W + fcoord(coords, j, c)];
                mm *= en.mant;
                ks += en.expo;
            }
            wemit[i] = mm != 0.0f ? mm * exp2i(max(ks - kmx[t], -200)) : 0.0f;
        }
        __syncthreads();

        // Backward through timestep t's chain from CUR into bv[0..C+4]:
        // bv0 in(CB) bv1 in(DT) bv2+c in(BL c) bv2+C in(ED) bv3+C in(EM).
        auto backward_timestep = [&](int t) {
            const SVec out_v = vec(CUR);
            const long n1 = (long)(t + 1) * S, n0 = (long)t * S;
            cta_emit<HB>(out_v, vec(BV + 3 + C), wemit + (long)t * S, S, n1);
            const SVec e3 = vec(BV + 3 + C), e2 = vec(BV + 2 + C);
            FOR_STATES(n0, S, i, e, j) {
                const int dc = a.dye[e];
                float v = pf * e3.A[i];
                if (dc < 0) {
                    v = fmaf(qf, e3.A[i + S], v);
                } else {
                    const float tot = (float)a.tot[e];
                    const int nc = fcoord(coords, (int)j, dc);
                    if ((float)nc < tot) v = fmaf(qf * (1.0f - (float)nc / tot), e3.A[i + S], v);
                    if (nc >= 1) v = fmaf(qf * ((float)nc / tot), e3.A[i + S - st[dc]], v);
                }
                e2.A[i] = v;
                if (HB) e2.B[i] = e3.B[i];
            }
            if (threadIdx.x == 0) *e2.pd = *e3.pd;
            __syncthreads();
            for (int c = C - 1; c >= 0; c--)
                cta_binomial<HB>(vec(BV + 3 + c), vec(BV + 2 + c), coords, S, t, c, W[c], st[c], M.bleach[c], true);
            const float pdt = M.p_det[t - 1];
            const SVec b2 = vec(BV + 2), b1 = vec(BV + 1), b0 = vec(BV);
            const float pd2 = *b2.pd;
            for (long i = threadIdx.x; i < n0; i += blockDim.x) {
                b1.A[i] = fmaf(1.0f - pdt, b2.A[i], pdt * pd2);
                if (HB) b1.B[i] = fmaf(1.0f - pdt, b2.B[i], pdt * pd2);
            }
            if (threadIdx.x == 0) *b1.pd = pd2;
            __syncthreads();
            for (long i = threadIdx.x; i < n0; i += blockDim.x) {
                if (HB) {
                    b0.A[i] = fmaf(m.p_cb, b1.B[i], (1.0f - m.p_cb) * b1.A[i]);
                    b0.B[i] = b1.B[i];
                } else {
                    b0.A[i] = (1.0f - m.p_cb) * b1.A[i];
                }
            }
            if (threadIdx.x == 0) *b0.pd = *b1.pd;
            __syncthreads();
        };
        // t = 0: d0 in(IB) d1+c in(DD c) d1+C in(EM0), from CUR.
        auto backward_t0 = [&]() {
            cta_emit<HB>(vec(CUR), vec(BV + 1 + C), wemit, S, S);
            for (int c = C - 1; c >= 0; c--)
                cta_binomial<HB>(vec(BV + 2 + c), vec(BV + 1 + c), coords, S, 1, c, W[c], st[c], M.dud[c], true);
            const SVec b1 = vec(BV + 1), b0 = vec(BV);
            for (int j = threadIdx.x; j < S; j += blockDim.x) {
                if (HB) {
                    b0.A[j] = fmaf(m.p_ib, b1.B[j], (1.0f - m.p_ib) * b1.A[j]);
                    b0.B[j] = b1.B[j];
                } else {
                    b0.A[j] = (1.0f - m.p_ib) * b1.A[j];
                }
            }
            if (threadIdx.x == 0) *b0.pd = *b1.pd;
            __syncthreads();
        };
        auto copy_vec = [&](const SVec& src, const SVec& dst, long n, float scale) {
            for (long i = threadIdx.x; i < n; i += blockDim.x) {
                dst.A[i] = src.A[i] * scale;
                if (HB) dst.B[i] = src.B[i] * scale;
            }
            if (threadIdx.x == 0) *dst.pd = *src.pd * scale;
            __syncthreads();
        };

        // ---- backward pass with checkpoints cp[t] (input of timestep t's chain)
        {
            const SVec cur = vec(CUR);
            for (long i = threadIdx.x; i < cap; i += blockDim.x) {
                cur.A[i] = 1.0f;
                if (HB) cur.B[i] = 1.0f;
            }
            if (threadIdx.x == 0) {
                *cur.pd = 1.0f;
                Eb[T] = 0;
            }
            __syncthreads();
            for (int t = T - 1; t >= 1; t--) {
                backward_timestep(t);
                const long n0 = (long)t * S;
                const SVec b0 = vec(BV);
                float mx = 0.f;
                for (long i = threadIdx.x; i < n0; i += blockDim.x) {
                    mx = fmaxf(mx, b0.A[i]);
                    if (HB) mx = fmaxf(mx, b0.B[i]);
                }
                if (threadIdx.x == 0) mx = fmaxf(mx, *b0.pd);
                cta_reduce<true>(&mx, 1, red, rout);
                int k = 0;
                if (rout[0] > 0.f) frexpf(rout[0], &k);
                const float sc = exp2i(-k);
                copy_vec(b0, gvec(t), n0, sc);
                copy_vec(b0, vec(CUR), n0, sc);
                if (threadIdx.x == 0) Eb[t] = Eb[t + 1] + kmx[t] + k;
                __syncthreads();
            }
            backward_t0();
            if (threadIdx.x == 0) Eb[0] = Eb[1] + kmx[0];
            __syncthreads();
        }
        const float Ps = vec(BV).A[S - 1];
        if (!(Ps > 0.0f)) {
            if (threadIdx.x == 0 && a.logp) a.logp[ro] = -INFINITY;
            __syncthreads();
            continue;
        }
        int EP;
        const float Pm = frexpf(Ps, &EP);
        EP += Eb[0];
        if (threadIdx.x == 0 && a.logp) a.logp[ro] = log((double)Pm) + (double)EP * 0.69314718055994530942;
        auto scale_of = [&](int Ea, int Ebc) { return ldexp(1.0 / (double)Pm, Ea + Ebc - EP); };

        // emission statistics of emission t from the buckets (thread 0, FP64)
        auto emis_add = [&](int t, const SVec& f, const SVec& b, double sc) {
            if (threadIdx.x == 0) {
                const double* x = a.rads + ((long)r * T + t) * C;
                const double gd = (double)(*f.pd * *b.pd) * sc;
                int k = 0;
                for (int c = 0; c < C; c++)
                    for (int n = 0; n < W[c]; n++, k++) {
                        const double gs = (double)ebk[k] * sc + (n == 0 ? gd : 0.0);
                        acc[fs_emis(T, C, 0, c, n)] += gs;
                        acc[fs_emis(T, C, 1, c, n)] += gs * x[c];
                        acc[fs_emis(T, C, 2, c, n)] += gs * x[c] * x[c];
                    }
            }
        };
        // ---- forward sweep with the expected counts
        int fa = F0, fb = F1;
        int Ea = 0;
        float part[FIT_MAXTERMS];
        {
            // t = 0 (the backward vectors of timestep 0 are still in bv)
            const SVec al = vec(fa);
            for (long i = threadIdx.x; i < S; i += blockDim.x) {
                al.A[i] = (i == S - 1) ? 1.0f : 0.0f;
                if (HB) al.B[i] = 0.0f;
            }
            if (threadIdx.x == 0) *al.pd = 0.0f;
            __syncthreads();
            const double sc = scale_of(Ea, Eb[0]);
            for (int k = 0; k < FIT_MAXTERMS; k++) part[k] = 0.f;
            // initial block EM and transition
            for (int j = threadIdx.x; j < S; j += blockDim.x) {
                const float f = al.A[j];
                if (HB) part[0] = fmaf(f * m.p_ib, vec(BV + 1).B[j], part[0]);
                part[1] = fmaf(f, vec(BV).A[j], part[1]);
            }
            __syncthreads();
            for (int j = threadIdx.x; j < S; j += blockDim.x) {
                const float f = al.A[j];
                if (HB) al.B[j] = al.B[j] + m.p_ib * f;
                al.A[j] = (1.0f - m.p_ib) * f;
            }
            __syncthreads();
            for (int c = 0; c < C; c++) {
                const SVec f = vec(fa), b = vec(BV + 1 + c), nb = vec(BV + 2 + c);
                float n32 = 0.f, d32 = 0.f;
                for (int i = threadIdx.x; i < S; i += blockDim.x) {
                    const int from = fcoord(coords, i, c);
                    if (from < 1) continue;
                    d32 = fmaf(f.A[i] * b.A[i], (float)from, d32);
                    if (HB) d32 = fmaf(f.B[i] * b.B[i], (float)from, d32);
                    for (int to = 0; to < from; to++) {
                        const float p = M.dud[c][from * (from + 1) / 2 + to];
                        const long kk = i - (long)(from - to) * st[c];
                        n32 = fmaf(f.A[i] * p * nb.A[kk], (float)(from - to), n32);
                        if (HB) n32 = fmaf(f.B[i] * p * nb.B[kk], (float)(from - to), n32);
                    }
                }
                part[2 + 2 * c] = n32;
                part[3 + 2 * c] = d32;
                __syncthreads();
                cta_binomial<HB>(vec(fa), vec(fb), coords, S, 1, c, W[c], st[c], M.dud[c], false);
                const int tmp = fa;
                fa = fb;
                fb = tmp;
            }
            const int nt = 2 + 2 * C;
            cta_reduce<false>(part, nt, red, rout);
            if (threadIdx.x == 0) {
                acc[FS_IB_NUM] += (double)rout[0] * sc;
                acc[FS_IB_DEN] += (double)rout[1] * sc;
                for (int c = 0; c < C; c++) {
                    acc[fs_dud_num(T, c)] += (double)rout[2 + 2 * c] * sc;
                    acc[fs_dud_den(T, c)] += (double)rout[3 + 2 * c] * sc;
                }
            }
            if (a.emission) {
                cta_emission_buckets<HB>(vec(fa), vec(BV + 1 + C), vec(fb).A, S, S, C, W, coords, ebk);
                emis_add(0, vec(fa), vec(BV + 1 + C), sc);
            }
            // emission 0 and rescale
            cta_emit<HB>(vec(fa), vec(fa), wemit, S, S);
            const SVec al2 = vec(fa);
            float tot = 0.f;
            for (int j = threadIdx.x; j < S; j += blockDim.x) {
                tot += al2.A[j];
                if (HB) tot += al2.B[j];
            }
            if (threadIdx.x == 0) tot += *al2.pd;
            cta_reduce<false>(&tot, 1, red, rout);
            int k = 0;
            if (rout[0] > 0.f) frexpf(rout[0], &k);
            Ea += kmx[0];
            copy_vec(al2, al2, S, exp2i(-k));
            Ea += k;
        }
        for (int t = 1; t < T; t++) {
            // backward vectors of timestep t from checkpoint t + 1
            {
                const long nn = (long)(t + 1) * S;
                if (t + 1 == T) {
                    const SVec cur = vec(CUR);
                    for (long i = threadIdx.x; i < cap; i += blockDim.x) {
                        cur.A[i] = 1.0f;
                        if (HB) cur.B[i] = 1.0f;
                    }
                    if (threadIdx.x == 0) *cur.pd = 1.0f;
                    __syncthreads();
                } else {
                    copy_vec(gvec(t + 1), vec(CUR), nn, 1.0f);
                }
            }
            backward_timestep(t);
            const double sc = scale_of(Ea, Eb[t + 1] + kmx[t]);
            const long n0 = (long)t * S;
            for (int k = 0; k < FIT_MAXTERMS; k++) part[k] = 0.f;
            // cyclic block EM and transition
            {
                const SVec al = vec(fa), b0 = vec(BV), b1 = vec(BV + 1);
                for (long i = threadIdx.x; i < n0; i += blockDim.x) {
                    const float f = al.A[i];
                    if (HB) part[0] = fmaf(f * m.p_cb, b1.B[i], part[0]);
                    part[1] = fmaf(f, b0.A[i], part[1]);
                }
                __syncthreads();
                for (long i = threadIdx.x; i < n0; i += blockDim.x) {
                    const float f = al.A[i];
                    if (HB) al.B[i] = al.B[i] + m.p_cb * f;
                    al.A[i] = (1.0f - m.p_cb) * f;
                }
                __syncthreads();
            }
            // detach EM (skipping each slice's all-zero state) and transition
            float pd2 = 0.f;
            {
                const SVec al = vec(fa), b1 = vec(BV + 1), b2 = vec(BV + 2);
                const float pdt = M.p_det[t - 1];
                pd2 = *b2.pd;
                float fs = 0.f, fbv = 0.f, all = 0.f;
                FOR_STATES(n0, S, i, e, j) {
                    const float f = al.A[i];
                    all += f;
                    if (j != 0) {
                        fs += f;
                        fbv = fmaf(f, b1.A[i], fbv);
                    }
                    if (HB) {
                        const float g = al.B[i];
                        all += g;
                        if (j != 0) {
                            fs += g;
                            fbv = fmaf(g, b1.B[i], fbv);
                        }
                    }
                }
                part[2] = fs * pdt;
                part[3] = fbv;
                part[4] = all;
                cta_reduce<false>(part + 2, 3, red, rout);
                const float allsum = rout[2];
                part[2] = 0.f;  // reduced below from rout
                const float red_fs = rout[0], red_fb = rout[1];
                for (long i = threadIdx.x; i < n0; i += blockDim.x) {
                    al.A[i] *= 1.0f - pdt;
                    if (HB) al.B[i] *= 1.0f - pdt;
                }
                if (threadIdx.x == 0) {
                    *al.pd = *al.pd + pdt * allsum;
                    acc[fs_det_x(t - 1)] += (double)red_fs * (double)pd2 * sc;
                    acc[fs_det_n(t - 1)] += (double)red_fb * sc;
                }
                __syncthreads();
            }
            // bleach per channel
            for (int c = 0; c < C; c++) {
                const SVec f = vec(fa), b = vec(BV + 2 + c), nb = vec(BV + 3 + c);
                float n32 = 0.f, d32 = 0.f;
                FOR_STATES(n0, S, i, e, j) {
                    const int from = fcoord(coords, (int)j, c);
                    if (from < 1) continue;
                    d32 = fmaf(f.A[i] * b.A[i], (float)from, d32);
                    if (HB) d32 = fmaf(f.B[i] * b.B[i], (float)from, d32);
                    for (int to = 0; to < from; to++) {
                        const float p = M.bleach[c][from * (from + 1) / 2 + to];
                        const long kk = i - (long)(from - to) * st[c];
                        n32 = fmaf(f.A[i] * p * nb.A[kk], (float)(from - to), n32);
                        if (HB) n32 = fmaf(f.B[i] * p * nb.B[kk], (float)(from - to), n32);
                    }
                }
                part[6 + 2 * c] = n32;
                part[7 + 2 * c] = d32;
                __syncthreads();
                cta_binomial<HB>(vec(fa), vec(fb), coords, S, t, c, W[c], st[c], M.bleach[c], false);
                const int tmp = fa;
                fa = fb;
                fb = tmp;
            }
            // Edman EM (skipping each slice's all-zero state) and transition
            {
                const SVec al = vec(fa), e2 = vec(BV + 2 + C), e3 = vec(BV + 3 + C), an = vec(fb);
                float n32 = 0.f, d32 = 0.f;
                FOR_STATES(n0, S, i, e, j) {
                    if (j == 0) continue;
                    const float f = al.A[i];
                    n32 = fmaf(f * pf, e3.A[i], n32);
                    d32 = fmaf(f, e2.A[i], d32);
                }
                part[4] = n32;
                part[5] = d32;
                const long n1 = (long)(t + 1) * S;
                FOR_STATES(n1, S, i, e, j) {
                    float v = e < t ? pf * al.A[i] : 0.0f;
                    if (e >= 1) {
                        const int dc = a.dye[e - 1];
                        const float xin = al.A[i - S];
                        if (dc < 0) {
                            v = fmaf(qf, xin, v);
                        } else {
                            const float tot = (float)a.tot[e - 1];
                            const int nc = fcoord(coords, (int)j, dc);
                            if ((float)nc < tot) v = fmaf(qf * (1.0f - (float)nc / tot), xin, v);
                            if (nc + 1 < W[dc]) v = fmaf(qf * ((float)(nc + 1) / tot), al.A[i - S + st[dc]], v);
                        }
                    }
                    an.A[i] = v;
                    if (HB) an.B[i] = e < t ? al.B[i] : 0.0f;
                }
                if (threadIdx.x == 0) *an.pd = *al.pd;
                __syncthreads();
                const int tmp = fa;
                fa = fb;
                fb = tmp;
            }
            // the timestep's remaining terms: block (0, 1), Edman (4, 5),
            // bleach (6 ..)
            {
                float v[FIT_MAXTERMS];
                int nt = 0;
                v[nt++] = part[0];
                v[nt++] = part[1];
                v[nt++] = part[4];
                v[nt++] = part[5];
                for (int c = 0; c < C; c++) {
                    v[nt++] = part[6 + 2 * c];
                    v[nt++] = part[7 + 2 * c];
                }
                cta_reduce<false>(v, nt, red, rout);
                if (threadIdx.x == 0) {
                    acc[FS_CB_NUM] += (double)rout[0] * sc;
                    acc[FS_CB_DEN] += (double)rout[1] * sc;
                    acc[FS_EDMAN_NUM] += (double)rout[2] * sc;
                    acc[FS_EDMAN_DEN] += (double)rout[3] * sc;
                    for (int c = 0; c < C; c++) {
                        acc[fs_bleach_num(T, c)] += (double)rout[4 + 2 * c] * sc;
                        acc[fs_bleach_den(T, c)] += (double)rout[5 + 2 * c] * sc;
                    }
                }
            }
            if (a.emission) {
                cta_emission_buckets<HB>(vec(fa), vec(BV + 3 + C), vec(fb).A, (long)(t + 1) * S, S, C, W, coords,
                                         ebk);
                emis_add(t, vec(fa), vec(BV + 3 + C), sc);
            }
            // emission t and rescale
            {
                const long n1 = (long)(t + 1) * S;
                cta_emit<HB>(vec(fa), vec(fa), wemit + (long)t * S, S, n1);
                const SVec al = vec(fa);
                float tot = 0.f;
                for (long i = threadIdx.x; i < n1; i += blockDim.x) {
                    tot += al.A[i];
                    if (HB) tot += al.B[i];
                }
                if (threadIdx.x == 0) tot += *al.pd;
                cta_reduce<false>(&tot, 1, red, rout);
                int k = 0;
                if (rout[0] > 0.f) frexpf(rout[0], &k);
                Ea += kmx[t];
                copy_vec(al, al, n1, exp2i(-k));
                Ea += k;
            }
        }
        __syncthreads();
    }
    // this CTA's sums, slot-major [nslots][grid]
    for (int k = threadIdx.x; k < a.nslots; k += blockDim.x) a.sums[(long)k * gridDim.x + blockIdx.x] = acc[k];
}

size_t wp_fit_cta_smem_bytes(int T, int C, int S, bool has_block, bool emission) {
    const long cap = (long)T * S;
    const long VS = (((has_block ? 2 : 1) * cap + 1) + 3) / 4 * 4;
    size_t b = sizeof(float) * ((size_t)(C + 8) * VS + (size_t)T * S) + sizeof(uint32_t) * S +
               sizeof(float) * (FIT_MAXTERMS * 32 + FIT_MAXTERMS) + sizeof(int) * (2 * WP_MAX_TIMESTEPS + 2) + 8 +
               sizeof(float) * FIT_EMIS_BUCKETS + sizeof(double) * fit_nslots(T, C, emission);
    return b;
}

long wp_fit_cta_ckpt_floats(int T, int S, bool has_block) {
    const long cap = (long)T * S;
    const long VS = (((has_block ? 2 : 1) * cap + 1) + 3) / 4 * 4;
    return (long)(T + 1) * VS;
}

cudaError_t wp_launch_fit_cta(bool has_block, int grid, size_t smem, cudaStream_t s, const FitArgs& a, float* ckpt,
                              long ck_stride) {
    if (has_block) {
        cudaFuncSetAttribute(wp_fit_cta_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        wp_fit_cta_kernel<true><<<grid, FIT_NT, smem, s>>>(a, ckpt, ck_stride);
    } else {
        cudaFuncSetAttribute(wp_fit_cta_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        wp_fit_cta_kernel<false><<<grid, FIT_NT, smem, s>>>(a, ckpt, ck_stride);
    }
    return cudaGetLastError();
}

int wp_fit_cta_ctas_per_sm(bool has_block, size_t smem) {
    int n = 0;
    if (has_block) {
        cudaFuncSetAttribute(wp_fit_cta_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, wp_fit_cta_kernel<true>, FIT_NT, smem);
    } else {
        cudaFuncSetAttribute(wp_fit_cta_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, wp_fit_cta_kernel<false>, FIT_NT, smem);
    }
    return n;
}

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

// Sum slots per thread (doubles): see fit_slot_*.
__host__ __device__ inline int fit_nslots(int T, int C) { return 6 + 2 * (T - 1) + 4 * C; }
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

int wp_fit_nslots(int T, int C) { return fit_nslots(T, C); }

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

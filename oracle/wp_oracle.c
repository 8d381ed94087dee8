/*
 * wp_oracle.c -- CPU FP64 restatement of whatprot's peptide HMM.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  See wp_oracle.h for the contract.
 * Every routine below restates one reference routine; the reference
 * file:line it follows is cited at each definition.  Paths are relative to
 * the reference project's cc_code/src/.
 *
 * Representation: a state vector is two dense FP64 tensors (normal and
 * broken-N) over an axis-aligned box of (Edman count, dye count per
 * channel), a detached-state scalar and an allow-detached flag, exactly as
 * hmm/state-vector/peptide-state-vector.{h,cc}.  Tensors are row-major over
 * their own box (tensor/tensor.cc:45-54).
 */
#include "wp_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORD_MAX (1 + WPO_MAX_CHANNELS)

/* ---------------------------------------------------------------- KDRange */
/* util/kd-range.cc:18-48 */
typedef struct {
    int n;
    unsigned min[ORD_MAX];
    unsigned max[ORD_MAX];
} krange;

static krange kr_intersect(const krange* a, const krange* b) {
    krange r;
    r.n = a->n;
    for (int i = 0; i < a->n; i++) {
        r.min[i] = a->min[i] > b->min[i] ? a->min[i] : b->min[i];
        r.max[i] = a->max[i] < b->max[i] ? a->max[i] : b->max[i];
    }
    return r;
}

static int kr_empty(const krange* r) {
    for (int i = 0; i < r->n; i++)
        if (r->min[i] >= r->max[i]) return 1;
    return 0;
}

static int kr_includes_zero(const krange* r) {
    for (int i = 0; i < r->n; i++) {
        if (r->min[i] > 0) return 0;
        if (r->max[i] <= 0) return 0;
    }
    return 1;
}

/* Row-major odometer over a box (tensor/base-tensor-iterator.h:68-90). */
typedef struct {
    krange r;
    unsigned loc[ORD_MAX];
    int done;
} kiter;

static void kit_begin(kiter* it, const krange* r) {
    it->r = *r;
    it->done = kr_empty(r);
    for (int i = 0; i < r->n; i++) it->loc[i] = r->min[i];
}

static void kit_next(kiter* it) {
    for (int o = it->r.n - 1; o >= 0; o--) {
        it->loc[o]++;
        if (it->loc[o] < it->r.max[o]) return;
        it->loc[o] = it->r.min[o];
    }
    it->done = 1;
}

/* ----------------------------------------------------------------- Tensor */
/* tensor/tensor.cc:45-54 (strides from the box extents, zero-filled). */
typedef struct {
    krange range;
    long strides[ORD_MAX];
    long size;
    double* v;
} tensor;

static void tensor_init(tensor* t, const krange* r) {
    t->range = *r;
    long size = 1;
    for (int i = r->n - 1; i >= 0; i--) {
        t->strides[i] = size;
        size *= (long)(r->max[i] - r->min[i]);
    }
    t->size = size;
    t->v = (double*)calloc(size > 0 ? size : 1, sizeof(double));
}

static void tensor_free(tensor* t) {
    free(t->v);
    t->v = NULL;
}

static long tensor_index(const tensor* t, const unsigned* loc) {
    long idx = 0;
    for (int i = 0; i < t->range.n; i++)
        idx += t->strides[i] * (long)(loc[i] - t->range.min[i]);
    return idx;
}

/* tensor/tensor.cc:111-121 */
static double tensor_sum(const tensor* t, const krange* r) {
    double total = 0.0;
    kiter it;
    for (kit_begin(&it, r); !it.done; kit_next(&it))
        total += t->v[tensor_index(t, it.loc)];
    return total;
}

/* ------------------------------------------------------------ StateVector */
/* hmm/state-vector/peptide-state-vector.cc:32-58 */
typedef struct {
    tensor a;  /* tensor */
    tensor b;  /* broken_n_tensor */
    krange range;
    double pd; /* p_detached */
    int allow; /* allow_detached */
} psv;

static psv* psv_new(const krange* r) {
    psv* s = (psv*)calloc(1, sizeof(psv));
    tensor_init(&s->a, r);
    tensor_init(&s->b, r);
    s->range.n = 0;
    s->pd = 0.0;
    s->allow = 1;
    return s;
}

static void psv_free(psv* s) {
    if (!s) return;
    tensor_free(&s->a);
    tensor_free(&s->b);
    free(s);
}

static double psv_sum(const psv* s) {
    return tensor_sum(&s->a, &s->range) + tensor_sum(&s->b, &s->range) + s->pd;
}

/* Multiply every stored value by 2^-k (exact; used for rescaling). */
static void psv_scale_pow2(psv* s, int k) {
    for (long i = 0; i < s->a.size; i++) s->a.v[i] = ldexp(s->a.v[i], -k);
    for (long i = 0; i < s->b.size; i++) s->b.v[i] = ldexp(s->b.v[i], -k);
    s->pd = ldexp(s->pd, -k);
}

/* ----------------------------------------------------------- Model pieces */
/* parameterization/model/channel-model.h:35-54 (adjusted_mu). */
double wpo_adjusted_mu(const wpo_model* m, int channel, const unsigned* counts) {
    double amu = m->mu[channel];
    amu *= (double)counts[channel];
    for (int c = 0; c < m->num_channels; c++) {
        if (c == channel) {
            if (counts[c] > 1) {
                amu *= m->flat_interactions[channel][c];
                amu *= pow(m->interactions[channel][c], counts[c] - 1);
            }
        } else {
            if (counts[c] > 0) {
                amu *= m->flat_interactions[channel][c];
                amu *= pow(m->interactions[channel][c], counts[c]);
            }
        }
    }
    return amu;
}

/* parameterization/model/channel-model.cc:35-37 */
double wpo_sigma(const wpo_model* m, int channel, double amu) {
    return sqrt(m->bg_sig[channel] * m->bg_sig[channel]
                + amu * m->sig[channel] * m->sig[channel]);
}

/* parameterization/model/channel-model.h:61-70 (pdf_helper). */
double wpo_pdf(const wpo_model* m, int channel, double observed,
               const unsigned* counts) {
    static const double pi = 3.141592653589793238;
    double amu = wpo_adjusted_mu(m, channel, counts);
    double offset = observed - amu;
    double s = wpo_sigma(m, channel, amu);
    return (1.0 / (s * sqrt(2.0 * pi))) * exp(-offset * offset / (2.0 * s * s));
}

/* parameterization/model/decaying-rate-model.cc:47-50 */
double wpo_p_detach_at(const wpo_model* m, unsigned t) {
    return m->p_detach + m->p_initial_detach
                                 * exp(-(double)t * m->p_initial_detach_decay);
}

/* common/dye-track.cc:26-43 */
void wpo_dye_track(int T, int C, const int16_t* seq, int length, int16_t* out) {
    int16_t cs[WPO_MAX_CHANNELS];
    memset(cs, 0, sizeof(cs));
    memset(out, 0, sizeof(int16_t) * T * C);
    for (int t = length - 1; t >= 0; t--) {
        int16_t dye = seq[t];
        if (dye != -1) cs[dye]++;
        if (t < T) memcpy(&out[t * C], cs, sizeof(int16_t) * C);
    }
}

/* common/dye-seq.cc:52-58: out-of-range positions read as -1. */
static int dye_at(const int16_t* seq, int length, unsigned i) {
    return (int)i < length ? seq[i] : -1;
}

/* hmm/step/peptide-emission.cc:50-163 */
void wpo_emission_range(const wpo_model* m, const double* rad, int t,
                        unsigned max_num_dyes, double dist_cutoff,
                        unsigned* out_min, unsigned* out_max) {
    int C = m->num_channels;
    if (dist_cutoff == DBL_MAX) {
        for (int c = 0; c < C; c++) {
            out_min[c] = 0;
            out_max[c] = max_num_dyes + 1;
        }
        return;
    }
    unsigned counts_lo[WPO_MAX_CHANNELS] = {0};
    unsigned counts_hi[WPO_MAX_CHANNELS] = {0};
    /* The reference iterates to a fixed point without a bound; for
     * intensities below about -0.5 mu the iteration cycles forever (e.g.
     * counts 0 -> max+1 -> 1 -> 0 ...).  Both this restatement and the CUDA
     * prep kernel stop after 1000 rounds, so they agree on
     * such inputs; on every input where the reference terminates they
     * perform the same iterations. */
    int did_change = 1;
    int rounds = 0;
    while (did_change && rounds < 1000) {
        did_change = 0;
        rounds++;
        for (int c = 0; c < C; c++) {
            double old_counts_hi_c = counts_hi[c];
            counts_hi[c] = 1;
            double mu1 = wpo_adjusted_mu(m, c, counts_hi);
            counts_hi[c] = (unsigned)old_counts_hi_c;
            double mu = wpo_adjusted_mu(m, c, counts_hi);
            double s = dist_cutoff * wpo_sigma(m, c, mu);
            unsigned new_cts = (unsigned)lround((rad[t * C + c] + s) / mu1);
            if (new_cts > max_num_dyes + 1) new_cts = max_num_dyes + 1;
            if (new_cts != counts_hi[c]) {
                did_change = 1;
                counts_hi[c] = new_cts;
            }
        }
    }
    for (int c = 0; c < C; c++) {
        unsigned cmin = max_num_dyes + 1;
        double old_lo = counts_lo[c];
        for (unsigned d = 0; d < max_num_dyes + 1; d++) {
            counts_lo[c] = d;
            double mu = wpo_adjusted_mu(m, c, counts_lo);
            double s = dist_cutoff * wpo_sigma(m, c, mu);
            if (mu + s > rad[t * C + c]) {
                cmin = d;
                break;
            }
        }
        out_min[c] = cmin;
        counts_lo[c] = (unsigned)old_lo;
        unsigned cmax = max_num_dyes + 1;
        double old_hi = counts_hi[c];
        for (unsigned d = cmin; d < max_num_dyes + 1; d++) {
            counts_hi[c] = d;
            double mu = wpo_adjusted_mu(m, c, counts_hi);
            double s = dist_cutoff * wpo_sigma(m, c, mu);
            if (mu - s > rad[t * C + c]) {
                cmax = d;
                break;
            }
        }
        out_max[c] = cmax;
        counts_hi[c] = (unsigned)old_hi;
    }
}

/* hmm/step/binomial-transition.cc:51-67 (reserve) and :69-75 (prob). */
static void binomial_table(double q, unsigned max_n, double* tab) {
    double p = (double)1 - q;
    tab[0] = 1.0;
    for (unsigned i = 1; i <= max_n; i++) {
        tab[i * (i + 1) / 2 + 0] = tab[(i - 1) * i / 2 + 0] * q;
        for (unsigned j = 1; j < i; j++)
            tab[i * (i + 1) / 2 + j] = tab[(i - 1) * i / 2 + j] * q
                                       + tab[(i - 1) * i / 2 + j - 1] * p;
        tab[i * (i + 1) / 2 + i] = tab[(i - 1) * i / 2 + i - 1] * p;
    }
}
#define BPROB(tab, from, to) ((tab)[(from) * ((from) + 1) / 2 + (to)])

/* ------------------------------------------------------------------ Steps */
enum { S_INIT_BLOCK, S_DUD, S_EMIT, S_CYC_BLOCK, S_DETACH, S_BLEACH, S_EDMAN };

typedef struct {
    int kind;
    int channel; /* binomial steps */
    int t;       /* emission timestep or detach timestep index */
    double p;    /* block p / detach p / edman p_fail / binomial q */
    const double* tab; /* binomial table */
    const tensor* ptsr; /* emission table (over the emission's own box) */
    /* block, detach, emission: r1 = pruned_range.
     * binomial: r1 = forward_range, r2 = backward_range.
     * edman: r1 = true_forward, r2 = safe_forward, r3 = true_backward,
     *        r4 = safe_backward. */
    krange r1, r2, r3, r4;
    int allow;   /* emission allow_detached */
    int det_fwd; /* detach detached_forward */
    int det_bwd; /* detach detached_backward */
} step;

typedef struct {
    int T, C;
    const wpo_model* m;
    const int16_t* seq;
    int length;
    int16_t track[WPO_MAX_TIMESTEPS * WPO_MAX_CHANNELS];
    int nsteps;
    step* steps;
    krange forward_range, backward_range;
    int empty;
    /* emission tables (RadiometryPrecomputations) and binomial tables */
    tensor ptsr[WPO_MAX_TIMESTEPS];
    krange emit_range[WPO_MAX_TIMESTEPS];
    double* dud_tab[WPO_MAX_CHANNELS];
    double* bleach_tab[WPO_MAX_CHANNELS];
    double p_detach[WPO_MAX_TIMESTEPS];
    const double* rad; /* the read, [T][C] */
} hmm;

/* Edman ranges (hmm/step/edman-transition.cc:28-60). */
static void edman_set_true_forward(step* s, const krange* r) {
    s->r1 = *r;
    s->r4 = *r;
    s->r4.max[0]++;
    for (int c = 0; c < s->r4.n - 1; c++)
        if (s->r4.min[1 + c] != 0) s->r4.min[1 + c]--;
}

static void edman_set_true_backward(step* s, const krange* r) {
    s->r3 = *r;
    s->r2 = *r;
    if (s->r2.min[0] != 0) s->r2.min[0]--;
    for (int c = 0; c < s->r2.n - 1; c++) s->r2.max[1 + c]++;
}

static void prune_forward(step* s, krange* range, int* allow_detached) {
    switch (s->kind) {
    case S_INIT_BLOCK:
    case S_CYC_BLOCK: /* hmm/step/block-transition.cc:24-26 */
        s->r1 = *range;
        break;
    case S_DUD:
    case S_BLEACH: /* hmm/step/binomial-transition.cc:77-81 */
        s->r1 = *range;
        range->min[1 + s->channel] = 0;
        s->r2 = *range;
        break;
    case S_EMIT: /* hmm/step/peptide-emission.cc:198-203 */
        s->r1 = kr_intersect(&s->r1, range);
        *range = s->r1;
        s->allow = kr_includes_zero(&s->r1);
        *allow_detached = s->allow;
        break;
    case S_DETACH: /* hmm/step/detach-transition.cc:24-28 */
        s->r1 = *range;
        s->det_fwd = *allow_detached;
        *allow_detached = 1;
        break;
    case S_EDMAN: /* hmm/step/edman-transition.cc:50-53 */
        edman_set_true_forward(s, range);
        *range = s->r4;
        break;
    }
}

static void prune_backward(step* s, krange* range, int* allow_detached) {
    switch (s->kind) {
    case S_INIT_BLOCK:
    case S_CYC_BLOCK: /* hmm/step/block-transition.cc:28-31 */
        s->r1 = kr_intersect(&s->r1, range);
        *range = s->r1;
        break;
    case S_DUD:
    case S_BLEACH: /* hmm/step/binomial-transition.cc:83-89 */
        s->r2 = kr_intersect(&s->r2, range);
        *range = s->r2;
        range->max[1 + s->channel] = UINT32_MAX;
        s->r1 = kr_intersect(&s->r1, range);
        *range = s->r1;
        break;
    case S_EMIT: /* hmm/step/peptide-emission.cc:205-210 */
        s->r1 = kr_intersect(&s->r1, range);
        *range = s->r1;
        s->allow = kr_includes_zero(&s->r1);
        *allow_detached = s->allow;
        break;
    case S_DETACH: /* hmm/step/detach-transition.cc:30-34: the reference
                      assigns the (non-null) pointer, so this is true. */
        s->r1 = kr_intersect(&s->r1, range);
        *range = s->r1;
        s->det_bwd = 1;
        break;
    case S_EDMAN: /* hmm/step/edman-transition.cc:55-60 */
        *range = kr_intersect(&s->r4, range);
        edman_set_true_backward(s, range);
        *range = kr_intersect(&s->r2, &s->r1);
        edman_set_true_forward(s, range);
        break;
    }
}

/* RadiometryPrecomputations / PeptideEmission ctor
 * (hmm/precomputations/radiometry-precomputations.cc:20-29,
 *  hmm/step/peptide-emission.cc:39-181). */
static void build_emissions(hmm* h, const double* rad, unsigned max_num_dyes,
                            double dist_cutoff) {
    int C = h->C;
    for (int t = 0; t < h->T; t++) {
        unsigned lo[WPO_MAX_CHANNELS], hi[WPO_MAX_CHANNELS];
        wpo_emission_range(h->m, rad, t, max_num_dyes, dist_cutoff, lo, hi);
        krange pr;
        pr.n = 1 + C;
        pr.min[0] = 0;
        pr.max[0] = (unsigned)t + 1;
        for (int c = 0; c < C; c++) {
            pr.min[1 + c] = lo[c];
            pr.max[1 + c] = hi[c];
        }
        h->emit_range[t] = pr;
        krange tr;
        tr.n = C;
        for (int c = 0; c < C; c++) {
            tr.min[c] = lo[c];
            tr.max[c] = hi[c];
        }
        tensor_init(&h->ptsr[t], &tr);
        kiter it;
        for (kit_begin(&it, &tr); !it.done; kit_next(&it)) {
            double v = 1.0;
            for (int c = 0; c < C; c++)
                v *= wpo_pdf(h->m, c, rad[t * C + c], it.loc);
            h->ptsr[t].v[tensor_index(&h->ptsr[t], it.loc)] = v;
        }
    }
}

/* PeptideHMM ctor (hmm/hmm/peptide-hmm.cc:33-84), with
 * DyeSeqPrecomputations (hmm/precomputations/dye-seq-precomputations.cc:20-39)
 * and UniversalPrecomputations (universal-precomputations.cc:23-59). */
static void hmm_build(hmm* h, const wpo_model* m, int T, const int16_t* seq,
                      int length, const double* rad, unsigned max_num_dyes,
                      double dist_cutoff) {
    memset(h, 0, sizeof(*h));
    int C = m->num_channels;
    h->T = T;
    h->C = C;
    h->m = m;
    h->seq = seq;
    h->length = length;
    h->rad = rad;
    wpo_dye_track(T, C, seq, length, h->track);
    for (int c = 0; c < C; c++) {
        h->dud_tab[c] = (double*)calloc((max_num_dyes + 1) * (max_num_dyes + 2) / 2,
                                        sizeof(double));
        h->bleach_tab[c] = (double*)calloc((max_num_dyes + 1) * (max_num_dyes + 2) / 2,
                                           sizeof(double));
        binomial_table(m->p_dud[c], max_num_dyes, h->dud_tab[c]);
        binomial_table(m->p_bleach[c], max_num_dyes, h->bleach_tab[c]);
    }
    for (int t = 0; t < T; t++) h->p_detach[t] = wpo_p_detach_at(m, (unsigned)t);
    build_emissions(h, rad, max_num_dyes, dist_cutoff);

    h->nsteps = 1 + C + 1 + (T - 1) * (3 + C + 1);
    h->steps = (step*)calloc(h->nsteps, sizeof(step));
    int k = 0;
    step* s;
    s = &h->steps[k++];
    s->kind = S_INIT_BLOCK;
    s->p = m->p_initial_block;
    for (int c = 0; c < C; c++) {
        s = &h->steps[k++];
        s->kind = S_DUD;
        s->channel = c;
        s->p = m->p_dud[c];
        s->tab = h->dud_tab[c];
    }
    s = &h->steps[k++];
    s->kind = S_EMIT;
    s->t = 0;
    s->r1 = h->emit_range[0];
    s->ptsr = &h->ptsr[0];
    for (int t = 1; t < T; t++) {
        s = &h->steps[k++];
        s->kind = S_CYC_BLOCK;
        s->p = m->p_cyclic_block;
        s = &h->steps[k++];
        s->kind = S_DETACH;
        s->t = t - 1;
        s->p = h->p_detach[t - 1];
        for (int c = 0; c < C; c++) {
            s = &h->steps[k++];
            s->kind = S_BLEACH;
            s->channel = c;
            s->p = m->p_bleach[c];
            s->tab = h->bleach_tab[c];
        }
        s = &h->steps[k++];
        s->kind = S_EDMAN;
        s->p = m->p_edman_failure;
        s = &h->steps[k++];
        s->kind = S_EMIT;
        s->t = t;
        s->r1 = h->emit_range[t];
        s->ptsr = &h->ptsr[t];
    }

    krange range;
    range.n = 1 + C;
    range.min[0] = 0;
    range.max[0] = (unsigned)T;
    for (int c = 0; c < C; c++) {
        range.min[1 + c] = 0;
        range.max[1 + c] = 1 + (unsigned)h->track[c]; /* dye_track(0, c) */
    }
    int allow_detached = 0;
    for (int i = 0; i < h->nsteps; i++) {
        prune_forward(&h->steps[i], &range, &allow_detached);
        if (kr_empty(&range)) {
            h->empty = 1;
            return;
        }
    }
    h->backward_range = range;
    for (int i = h->nsteps - 1; i >= 0; i--) {
        prune_backward(&h->steps[i], &range, &allow_detached);
        if (kr_empty(&range)) {
            h->empty = 1;
            return;
        }
    }
    h->forward_range = range;
}

static void hmm_free(hmm* h) {
    for (int c = 0; c < h->C; c++) {
        free(h->dud_tab[c]);
        free(h->bleach_tab[c]);
    }
    for (int t = 0; t < h->T; t++) tensor_free(&h->ptsr[t]);
    free(h->steps);
}

/* Fiber transform along one channel axis (binomial-transition.cc:104-136). */
static void binomial_fwd_tensor(const step* s, const tensor* in, tensor* out,
                                double* flops) {
    int dim = 1 + s->channel;
    krange fibers = s->r2; /* iterate other coordinates over backward_range */
    fibers.min[dim] = 0;
    fibers.max[dim] = 1;
    unsigned to_min = s->r2.min[dim], to_max = s->r2.max[dim];
    unsigned fr_min = s->r1.min[dim], fr_max = s->r1.max[dim];
    kiter it;
    for (kit_begin(&it, &fibers); !it.done; kit_next(&it)) {
        unsigned loc[ORD_MAX];
        memcpy(loc, it.loc, sizeof(loc));
        for (unsigned to = to_min; to < to_max; to++) {
            double v_to = 0.0;
            unsigned from_min = to > fr_min ? to : fr_min;
            for (unsigned from = from_min; from < fr_max; from++) {
                loc[dim] = from;
                v_to += BPROB(s->tab, from, to) * in->v[tensor_index(in, loc)];
                if (flops) *flops += 2.0;
            }
            loc[dim] = to;
            out->v[tensor_index(out, loc)] = v_to;
        }
    }
}

static int g_count_broken = 0; /* visited-flops count only the normal tensor */

static psv* step_forward(const hmm* h, const step* s, const psv* in,
                         double* flops) {
    psv* out = NULL;
    kiter it;
    switch (s->kind) {
    case S_INIT_BLOCK:
    case S_CYC_BLOCK: { /* hmm/step/block-transition.cc:33-62 */
        out = psv_new(&s->r1);
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            double ta = in->a.v[tensor_index(&in->a, it.loc)];
            double tb = in->b.v[tensor_index(&in->b, it.loc)];
            out->a.v[tensor_index(&out->a, it.loc)] = (1 - s->p) * ta;
            out->b.v[tensor_index(&out->b, it.loc)] = tb + s->p * ta;
            if (flops && s->p != 0.0) *flops += 3.0;
        }
        out->range = s->r1;
        out->allow = in->allow;
        if (out->allow) out->pd = in->pd;
        break;
    }
    case S_DUD:
    case S_BLEACH: { /* hmm/step/binomial-transition.cc:91-102 */
        out = psv_new(&s->r2);
        binomial_fwd_tensor(s, &in->a, &out->a, flops);
        binomial_fwd_tensor(s, &in->b, &out->b, g_count_broken ? flops : NULL);
        out->range = s->r2;
        out->allow = in->allow;
        if (out->allow) out->pd = in->pd;
        break;
    }
    case S_EMIT: { /* hmm/step/peptide-emission.cc:212-243 */
        out = psv_new(&s->r1);
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            double prob = s->ptsr->v[tensor_index(s->ptsr, &it.loc[1])];
            out->a.v[tensor_index(&out->a, it.loc)] =
                    in->a.v[tensor_index(&in->a, it.loc)] * prob;
            if (flops) *flops += 1.0;
        }
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            double prob = s->ptsr->v[tensor_index(s->ptsr, &it.loc[1])];
            out->b.v[tensor_index(&out->b, it.loc)] =
                    in->b.v[tensor_index(&in->b, it.loc)] * prob;
        }
        if (s->allow) {
            unsigned zeros[ORD_MAX] = {0};
            double prob = s->ptsr->v[tensor_index(s->ptsr, zeros)];
            out->pd = in->pd * prob;
        }
        out->range = s->r1;
        out->allow = s->allow;
        break;
    }
    case S_DETACH: { /* hmm/step/detach-transition.cc:36-68 */
        out = psv_new(&s->r1);
        double sum = 0.0;
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            double value = in->a.v[tensor_index(&in->a, it.loc)];
            out->a.v[tensor_index(&out->a, it.loc)] = value * (1 - s->p);
            sum += value;
            if (flops) *flops += 2.0;
        }
        double sum_b = 0.0;
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            double value = in->b.v[tensor_index(&in->b, it.loc)];
            out->b.v[tensor_index(&out->b, it.loc)] = value * (1 - s->p);
            sum_b += value;
        }
        sum += sum_b;
        if (s->det_bwd) {
            if (s->det_fwd)
                out->pd = in->pd + s->p * sum;
            else
                out->pd = s->p * sum;
        }
        out->range = s->r1;
        out->allow = s->det_bwd;
        break;
    }
    case S_EDMAN: { /* hmm/step/edman-transition.cc:62-162 */
        const krange* tf = &s->r1;
        out = psv_new(&s->r4);
        long t_stride = out->a.strides[0];
        double pf = s->p;
        for (kit_begin(&it, tf); !it.done; kit_next(&it)) {
            double f_val = in->a.v[tensor_index(&in->a, it.loc)];
            long i = tensor_index(&out->a, it.loc);
            unsigned t = it.loc[0];
            int c = dye_at(h->seq, h->length, t);
            out->a.v[i] += pf * f_val;
            if (c == -1) {
                out->a.v[i + t_stride] += (1 - pf) * f_val;
            } else {
                unsigned c_idx = it.loc[1 + c];
                unsigned c_total = (unsigned)h->track[t * h->C + c];
                double ratio = (double)c_idx / (double)c_total;
                long c_stride = out->a.strides[1 + c];
                if (c_idx < c_total)
                    out->a.v[i + t_stride] += (1 - pf) * (1 - ratio) * f_val;
                if (c_idx > 0)
                    out->a.v[i + t_stride - c_stride] += (1 - pf) * ratio * f_val;
            }
            if (flops) *flops += 6.0;
        }
        for (kit_begin(&it, tf); !it.done; kit_next(&it))
            out->b.v[tensor_index(&out->b, it.loc)] =
                    in->b.v[tensor_index(&in->b, it.loc)];
        out->range = s->r3;
        out->allow = in->allow;
        if (out->allow) out->pd = in->pd;
        break;
    }
    }
    return out;
}

/* Exact power-of-two rescale so the state sums to [0.5, 1). */
static void rescale(psv* s, long* expo, double* flops) {
    double total = psv_sum(s);
    if (total > 0.0 && isfinite(total)) {
        int e;
        frexp(total, &e);
        psv_scale_pow2(s, e);
        *expo += e;
    }
    if (flops) {
        double states = 1.0;
        for (int i = 0; i < s->range.n; i++)
            states *= (double)(s->range.max[i] - s->range.min[i]);
        *flops += 2.0 * states;
    }
}

/* GenericHMM::probability (hmm/hmm/generic-hmm.h:41-55) with
 * PeptideHMM::probability (hmm/hmm/peptide-hmm.cc:94-100). */
static double hmm_probability(const hmm* h, double* log_p, double* flops) {
    if (h->empty) {
        if (log_p) *log_p = -INFINITY;
        return 0.0;
    }
    psv* in = psv_new(&h->forward_range);
    in->a.v[in->a.strides[0] - 1] = 1.0; /* initialize_from_start */
    long expo = 0;
    for (int i = 0; i < h->nsteps; i++) {
        psv* out = step_forward(h, &h->steps[i], in, flops);
        psv_free(in);
        in = out;
        if (h->steps[i].kind == S_EMIT) rescale(in, &expo, flops);
    }
    double s = psv_sum(in);
    psv_free(in);
    if (log_p) *log_p = (s > 0.0) ? log(s) + (double)expo * M_LN2 : -INFINITY;
    return ldexp(s, (int)expo);
}

double wpo_peptide_probability(const wpo_model* m, int num_timesteps,
                               const int16_t* seq, int length,
                               const double* rad, unsigned max_num_dyes,
                               double dist_cutoff, double* log_p,
                               double* visited_flops) {
    hmm h;
    hmm_build(&h, m, num_timesteps, seq, length, rad, max_num_dyes, dist_cutoff);
    if (visited_flops) *visited_flops = 0.0;
    double p = hmm_probability(&h, log_p, visited_flops);
    hmm_free(&h);
    return p;
}

int wpo_pruned_emission_boxes(const wpo_model* m, int num_timesteps,
                              const int16_t* seq, int length,
                              const double* rad, unsigned max_num_dyes,
                              double dist_cutoff, unsigned* lo, unsigned* hi) {
    hmm h;
    hmm_build(&h, m, num_timesteps, seq, length, rad, max_num_dyes, dist_cutoff);
    int empty = h.empty;
    if (!empty) {
        for (int i = 0; i < h.nsteps; i++) {
            const step* s = &h.steps[i];
            if (s->kind != S_EMIT) continue;
            for (int c = 0; c < h.C; c++) {
                lo[s->t * h.C + c] = s->r1.min[1 + c];
                hi[s->t * h.C + c] = s->r1.max[1 + c];
            }
        }
    }
    hmm_free(&h);
    return empty;
}

/* ------------------------------------------------------ Backward / EM */
/* binomial-transition.cc:151-183 */
static void binomial_bwd_tensor(const step* s, const tensor* in, tensor* out) {
    int dim = 1 + s->channel;
    krange fibers = s->r1; /* iterate other coordinates over forward_range */
    fibers.min[dim] = 0;
    fibers.max[dim] = 1;
    int from_min = (int)s->r1.min[dim], from_max = (int)s->r1.max[dim];
    int to_min = (int)s->r2.min[dim];
    int to_cap = (int)s->r2.max[dim] - 1;
    kiter it;
    for (kit_begin(&it, &fibers); !it.done; kit_next(&it)) {
        unsigned loc[ORD_MAX];
        memcpy(loc, it.loc, sizeof(loc));
        for (int from = from_max - 1; from >= from_min; from--) {
            double v_from = 0.0;
            int to_max = from < to_cap ? from : to_cap;
            for (int to = to_min; to <= to_max; to++) {
                loc[dim] = (unsigned)to;
                v_from += BPROB(s->tab, from, to) * in->v[tensor_index(in, loc)];
            }
            loc[dim] = (unsigned)from;
            out->v[tensor_index(out, loc)] = v_from;
        }
    }
}

static psv* step_backward(const hmm* h, const step* s, const psv* in) {
    psv* out = NULL;
    kiter it;
    switch (s->kind) {
    case S_INIT_BLOCK:
    case S_CYC_BLOCK: { /* hmm/step/block-transition.cc:64-93 */
        out = psv_new(&s->r1);
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            double ta = in->a.v[tensor_index(&in->a, it.loc)];
            double tb = in->b.v[tensor_index(&in->b, it.loc)];
            out->a.v[tensor_index(&out->a, it.loc)] = s->p * tb + (1 - s->p) * ta;
            out->b.v[tensor_index(&out->b, it.loc)] = tb;
        }
        out->range = s->r1;
        out->allow = in->allow;
        if (out->allow) out->pd = in->pd;
        break;
    }
    case S_DUD:
    case S_BLEACH: { /* hmm/step/binomial-transition.cc:138-149 */
        out = psv_new(&s->r1);
        binomial_bwd_tensor(s, &in->a, &out->a);
        binomial_bwd_tensor(s, &in->b, &out->b);
        out->range = s->r1;
        out->allow = in->allow;
        if (out->allow) out->pd = in->pd;
        break;
    }
    case S_EMIT: /* emission is its own transpose (peptide-emission.cc:250-253) */
        out = step_forward(h, s, in, NULL);
        break;
    case S_DETACH: { /* hmm/step/detach-transition.cc:70-103 */
        out = psv_new(&s->r1);
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            long o = tensor_index(&out->a, it.loc);
            out->a.v[o] = (1 - s->p) * in->a.v[tensor_index(&in->a, it.loc)];
            if (s->det_bwd) out->a.v[o] += s->p * in->pd;
        }
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            long o = tensor_index(&out->b, it.loc);
            out->b.v[o] = (1 - s->p) * in->b.v[tensor_index(&in->b, it.loc)];
            if (s->det_bwd) out->b.v[o] += s->p * in->pd;
        }
        if (s->det_fwd) out->pd = s->det_bwd ? in->pd : 0.0;
        out->range = s->r1;
        out->allow = s->det_fwd;
        break;
    }
    case S_EDMAN: { /* hmm/step/edman-transition.cc:164-277 */
        const krange* tb = &s->r3;
        out = psv_new(&s->r2);
        long t_stride = out->a.strides[0];
        double pf = s->p;
        for (kit_begin(&it, tb); !it.done; kit_next(&it)) {
            double f_val = in->a.v[tensor_index(&in->a, it.loc)];
            long i = tensor_index(&out->a, it.loc);
            unsigned t = it.loc[0];
            out->a.v[i] += pf * f_val;
            if (t > 0) {
                int c = dye_at(h->seq, h->length, t - 1);
                if (c == -1) {
                    out->a.v[i - t_stride] += (1 - pf) * f_val;
                } else {
                    unsigned c_total = (unsigned)h->track[(t - 1) * h->C + c];
                    long c_stride = out->a.strides[1 + c];
                    unsigned c_idx = it.loc[1 + c];
                    if (c_idx < c_total) {
                        double ratio = (double)c_idx / (double)c_total;
                        out->a.v[i - t_stride] += (1 - pf) * (1 - ratio) * f_val;
                    }
                    c_idx = it.loc[1 + c] + 1;
                    if (c_idx > 0) {
                        double ratio = (double)c_idx / (double)c_total;
                        out->a.v[i - t_stride + c_stride] += (1 - pf) * ratio * f_val;
                    }
                }
            }
        }
        for (kit_begin(&it, tb); !it.done; kit_next(&it))
            out->b.v[tensor_index(&out->b, it.loc)] =
                    in->b.v[tensor_index(&in->b, it.loc)];
        out->range = s->r1;
        out->allow = in->allow;
        if (out->allow) out->pd = in->pd;
        break;
    }
    }
    return out;
}

/* binomial-transition.cc:185-256 */
static void binomial_fit_tensor(const step* s, const tensor* f, const tensor* b,
                                const tensor* nb, double P, double* num,
                                double* den) {
    int dim = 1 + s->channel;
    krange fibers = s->r1;
    fibers.min[dim] = 0;
    fibers.max[dim] = 1;
    int from_min = (int)s->r1.min[dim], from_max = (int)s->r1.max[dim];
    int to_min = (int)s->r2.min[dim], to_max = (int)s->r2.max[dim];
    kiter it;
    for (kit_begin(&it, &fibers); !it.done; kit_next(&it)) {
        unsigned loc[ORD_MAX];
        memcpy(loc, it.loc, sizeof(loc));
        int lo = from_min > 1 ? from_min : 1;
        for (int from = from_max - 1; from >= lo; from--) {
            loc[dim] = (unsigned)from;
            double fv = f->v[tensor_index(f, loc)];
            double p_state = fv * b->v[tensor_index(b, loc)] / P;
            *den += p_state * (double)from;
            int hi = to_max < from ? to_max : from;
            for (int to = to_min; to < hi; to++) {
                loc[dim] = (unsigned)to;
                double p_tr = fv * BPROB(s->tab, from, to)
                              * nb->v[tensor_index(nb, loc)] / P;
                *num += p_tr * (double)(from - to);
            }
        }
    }
}

/* detach-transition.cc:121-166 (one tensor). */
static void detach_fit_tensor(const step* s, const tensor* f, const tensor* b,
                              double nb_pd, double P, wpo_fit_sums* sums) {
    double forward_sum = 0.0, fb_sum = 0.0;
    int skip_zero = kr_includes_zero(&s->r1);
    unsigned old_t = UINT32_MAX;
    kiter it;
    for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
        if (skip_zero && it.loc[0] != old_t) {
            old_t = it.loc[0];
            continue;
        }
        double fv = f->v[tensor_index(f, it.loc)];
        double bv = b->v[tensor_index(b, it.loc)];
        forward_sum += fv;
        fb_sum += fv * bv;
    }
    sums->detach_x[s->t] += forward_sum * s->p * nb_pd / P;
    sums->detach_n[s->t] += fb_sum / P;
}

static void step_improve_fit(const hmm* h, const step* s, const psv* fw,
                             const psv* bw, const psv* nbw, double P,
                             wpo_fit_sums* sums) {
    kiter it;
    switch (s->kind) {
    case S_INIT_BLOCK:
    case S_CYC_BLOCK: { /* block-transition.cc:95-116 */
        double* num = s->kind == S_INIT_BLOCK ? &sums->init_block_num : &sums->cyc_block_num;
        double* den = s->kind == S_INIT_BLOCK ? &sums->init_block_den : &sums->cyc_block_den;
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            double fv = fw->a.v[tensor_index(&fw->a, it.loc)];
            *num += fv * s->p * nbw->b.v[tensor_index(&nbw->b, it.loc)] / P;
            *den += fv * bw->a.v[tensor_index(&bw->a, it.loc)] / P;
        }
        break;
    }
    case S_DUD:
    case S_BLEACH: { /* dud-transition.cc:25-37, bleach-transition.cc:25-38 */
        int c = s->channel;
        double* num = s->kind == S_DUD ? &sums->dud_num[c] : &sums->bleach_num[c];
        double* den = s->kind == S_DUD ? &sums->dud_den[c] : &sums->bleach_den[c];
        binomial_fit_tensor(s, &fw->a, &bw->a, &nbw->a, P, num, den);
        binomial_fit_tensor(s, &fw->b, &bw->b, &nbw->b, P, num, den);
        break;
    }
    case S_EMIT: { /* peptide-emission.cc:255-260 is a no-op; the emission
                      statistics: posterior f * b / P of each state at this
                      emission, binned by each channel's dye count */
        const double* x = h->rad + (long)s->t * h->C;
        for (kit_begin(&it, &s->r1); !it.done; kit_next(&it)) {
            double g = fw->a.v[tensor_index(&fw->a, it.loc)] * bw->a.v[tensor_index(&bw->a, it.loc)] / P;
            g += fw->b.v[tensor_index(&fw->b, it.loc)] * bw->b.v[tensor_index(&bw->b, it.loc)] / P;
            for (int c = 0; c < h->C; c++) {
                const unsigned n = it.loc[1 + c];
                sums->emis_w[c][n] += g;
                sums->emis_x[c][n] += g * x[c];
                sums->emis_xx[c][n] += g * x[c] * x[c];
            }
        }
        {
            const double g = fw->pd * bw->pd / P;
            for (int c = 0; c < h->C; c++) {
                sums->emis_w[c][0] += g;
                sums->emis_x[c][0] += g * x[c];
                sums->emis_xx[c][0] += g * x[c] * x[c];
            }
        }
        break;
    }
    case S_DETACH:
        detach_fit_tensor(s, &fw->a, &bw->a, nbw->pd, P, sums);
        detach_fit_tensor(s, &fw->b, &bw->b, nbw->pd, P, sums);
        break;
    case S_EDMAN: { /* edman-transition.cc:279-325 */
        const krange* tf = &s->r1;
        int skip_zero = kr_includes_zero(tf);
        unsigned old_t = UINT32_MAX;
        for (kit_begin(&it, tf); !it.done; kit_next(&it)) {
            if (skip_zero && it.loc[0] != old_t) {
                old_t = it.loc[0];
                continue;
            }
            double fv = fw->a.v[tensor_index(&fw->a, it.loc)];
            double bv = bw->a.v[tensor_index(&bw->a, it.loc)];
            double nbv = nbw->a.v[tensor_index(&nbw->a, it.loc)];
            sums->edman_num += fv * s->p * nbv / P;
            sums->edman_den += fv * bv / P;
        }
        break;
    }
    }
}

/* GenericHMM::improve_fit (hmm/hmm/generic-hmm.h:60-109). */
double wpo_improve_fit(const wpo_model* m, int T, const int16_t* seq, int length,
                       const double* rad, unsigned max_num_dyes,
                       double dist_cutoff, wpo_fit_sums* sums, double* log_p) {
    hmm h;
    hmm_build(&h, m, T, seq, length, rad, max_num_dyes, dist_cutoff);
    if (log_p) hmm_probability(&h, log_p, NULL);
    if (h.empty) {
        hmm_free(&h);
        return 0.0;
    }
    psv** bsv = (psv**)calloc(h.nsteps + 1, sizeof(psv*));
    psv* fin = psv_new(&h.backward_range); /* initialize_from_finish */
    for (long i = 0; i < fin->a.size; i++) fin->a.v[i] = 1.0;
    for (long i = 0; i < fin->b.size; i++) fin->b.v[i] = 1.0;
    fin->pd = 1.0;
    bsv[h.nsteps] = fin; /* bsv[i] = backward state at the input of step i */
    for (int i = h.nsteps - 1; i >= 0; i--)
        bsv[i] = step_backward(&h, &h.steps[i], bsv[i + 1]);
    double P = bsv[0]->a.v[bsv[0]->a.strides[0] - 1]; /* source() */
    if (P != 0.0) {
        psv* fw = psv_new(&h.forward_range);
        fw->a.v[fw->a.strides[0] - 1] = 1.0;
        for (int i = 0; i < h.nsteps; i++) {
            step_improve_fit(&h, &h.steps[i], fw, bsv[i], bsv[i + 1], P, sums);
            psv* nx = step_forward(&h, &h.steps[i], fw, NULL);
            psv_free(fw);
            fw = nx;
        }
        psv_free(fw);
    }
    for (int i = 0; i <= h.nsteps; i++) psv_free(bsv[i]);
    free(bsv);
    hmm_free(&h);
    return P;
}

/* ------------------------------------------------------------- Classifier */
static unsigned max_num_dyes_of(int C, const int16_t* seqs, const int32_t* offsets,
                                int P, int T) {
    /* hmm/classifiers/hmm-classifier.cc:47-66: Dmax over all dye-seqs. */
    unsigned dmax = 0;
    int16_t track[WPO_MAX_TIMESTEPS * WPO_MAX_CHANNELS];
    for (int i = 0; i < P; i++) {
        wpo_dye_track(T, C, seqs + offsets[i], offsets[i + 1] - offsets[i], track);
        for (int c = 0; c < C; c++)
            if ((unsigned)track[c] > dmax) dmax = (unsigned)track[c];
    }
    return dmax;
}

static void classify_with_dmax(const wpo_model* m, int T, const int16_t* seqs,
                               const int32_t* offsets, const int32_t* ids,
                               const int32_t* counts, int P, const int32_t* cand,
                               int num_cand, const double* rad,
                               double dist_cutoff, unsigned dmax,
                               int32_t* out_id, double* out_score,
                               double* out_total) {
    /* classifiers/hmm-classifier.h:45-78 */
    int best_i = -1;
    double best_score = -1.0;
    double total_score = 0.0;
    int n = cand ? num_cand : P;
    for (int k = 0; k < n; k++) {
        int i = cand ? cand[k] : k;
        double score = wpo_peptide_probability(
                m, T, seqs + offsets[i], offsets[i + 1] - offsets[i], rad, dmax,
                dist_cutoff, NULL, NULL);
        total_score += score * counts[i];
        if (score > best_score) {
            best_score = score;
            best_i = i;
        }
    }
    double score = best_score, total = total_score;
    if (isnan(score / total)) {
        score = 0.0;
        total = 1.0;
    }
    *out_id = best_i >= 0 ? ids[best_i] : -1;
    *out_score = score;
    *out_total = total;
}

void wpo_classify_one(const wpo_model* m, int T, const int16_t* seqs,
                      const int32_t* offsets, const int32_t* ids,
                      const int32_t* counts, int P, const int32_t* cand,
                      int num_cand, const double* rad, double dist_cutoff,
                      int32_t* out_id, double* out_score, double* out_total) {
    unsigned dmax = max_num_dyes_of(m->num_channels, seqs, offsets, P, T);
    classify_with_dmax(m, T, seqs, offsets, ids, counts, P, cand, num_cand, rad,
                       dist_cutoff, dmax, out_id, out_score, out_total);
}

typedef struct {
    const wpo_model* m;
    int T;
    const int16_t* seqs;
    const int32_t* offsets;
    const int32_t* ids;
    const int32_t* counts;
    int P;
    const double* rads;
    int R;
    const int32_t* cand;
    const int32_t* cand_off;
    double dist_cutoff;
    unsigned dmax;
    int32_t* out_id;
    double* out_score;
    double* out_total;
    double* out_logp; /* loglik_all mode when non-NULL */
    int next;
    pthread_mutex_t lock;
} batch_job;

static void* batch_worker(void* arg) {
    batch_job* j = (batch_job*)arg;
    int C = j->m->num_channels;
    for (;;) {
        pthread_mutex_lock(&j->lock);
        int r = j->next++;
        pthread_mutex_unlock(&j->lock);
        if (r >= j->R) break;
        const double* rad = j->rads + (long)r * j->T * C;
        if (j->out_logp) {
            for (int i = 0; i < j->P; i++) {
                double lp;
                wpo_peptide_probability(j->m, j->T, j->seqs + j->offsets[i],
                                        j->offsets[i + 1] - j->offsets[i], rad,
                                        j->dmax, j->dist_cutoff, &lp, NULL);
                j->out_logp[(long)r * j->P + i] = lp;
            }
        } else {
            const int32_t* cand = NULL;
            int nc = 0;
            if (j->cand) {
                cand = j->cand + j->cand_off[r];
                nc = j->cand_off[r + 1] - j->cand_off[r];
            }
            classify_with_dmax(j->m, j->T, j->seqs, j->offsets, j->ids, j->counts,
                               j->P, cand, nc, rad, j->dist_cutoff, j->dmax,
                               &j->out_id[r], &j->out_score[r], &j->out_total[r]);
        }
    }
    return NULL;
}

static void run_batch(batch_job* j, int threads) {
    if (threads < 1) threads = 1;
    pthread_mutex_init(&j->lock, NULL);
    j->next = 0;
    pthread_t* th = (pthread_t*)calloc(threads, sizeof(pthread_t));
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, batch_worker, j);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&j->lock);
}

void wpo_classify_batch(const wpo_model* m, int T, const int16_t* seqs,
                        const int32_t* offsets, const int32_t* ids,
                        const int32_t* counts, int P, const double* rads, int R,
                        const int32_t* cand, const int32_t* cand_off,
                        double dist_cutoff, int threads, int32_t* out_id,
                        double* out_score, double* out_total) {
    batch_job j;
    memset(&j, 0, sizeof(j));
    j.m = m;
    j.T = T;
    j.seqs = seqs;
    j.offsets = offsets;
    j.ids = ids;
    j.counts = counts;
    j.P = P;
    j.rads = rads;
    j.R = R;
    j.cand = cand;
    j.cand_off = cand_off;
    j.dist_cutoff = dist_cutoff;
    j.dmax = max_num_dyes_of(m->num_channels, seqs, offsets, P, T);
    j.out_id = out_id;
    j.out_score = out_score;
    j.out_total = out_total;
    run_batch(&j, threads);
}

void wpo_loglik_all(const wpo_model* m, int T, const int16_t* seqs,
                    const int32_t* offsets, int P, const double* rads, int R,
                    double dist_cutoff, int threads, double* out_logp) {
    batch_job j;
    memset(&j, 0, sizeof(j));
    j.m = m;
    j.T = T;
    j.seqs = seqs;
    j.offsets = offsets;
    j.P = P;
    j.rads = rads;
    j.R = R;
    j.dist_cutoff = dist_cutoff;
    j.dmax = max_num_dyes_of(m->num_channels, seqs, offsets, P, T);
    j.out_logp = out_logp;
    run_batch(&j, threads);
}

/* ------------------------------------------------- Batched E-step (timing) */
typedef struct {
    const wpo_model* m;
    int T;
    const int16_t* seq;
    int length;
    const double* rads;
    int R;
    unsigned dmax;
    double dist_cutoff;
    int next;
    pthread_mutex_t lock;
    wpo_fit_sums* partial; /* one per thread */
    double* logp;          /* [R], may be NULL */
} fit_job;

typedef struct {
    fit_job* j;
    int id;
} fit_arg;

static void* fit_worker(void* arg) {
    fit_arg* a = (fit_arg*)arg;
    fit_job* j = a->j;
    int C = j->m->num_channels;
    for (;;) {
        pthread_mutex_lock(&j->lock);
        int r = j->next++;
        pthread_mutex_unlock(&j->lock);
        if (r >= j->R) break;
        double lp;
        wpo_improve_fit(j->m, j->T, j->seq, j->length, j->rads + (long)r * j->T * C,
                        j->dmax, j->dist_cutoff, &j->partial[a->id], &lp);
        if (j->logp) j->logp[r] = lp;
    }
    return NULL;
}

/* HMMFitter's per-iteration E-step loop (fitters/hmm-fitter.h:58-78) over
 * R reads on `threads` host threads; sums are added into *sums (per-thread
 * partial sums, combined in thread order). */
void wpo_improve_fit_batch(const wpo_model* m, int T, const int16_t* seq,
                           int length, const double* rads, int R,
                           double dist_cutoff, int threads, wpo_fit_sums* sums,
                           double* logp) {
    if (threads < 1) threads = 1;
    fit_job j;
    memset(&j, 0, sizeof(j));
    j.m = m;
    j.T = T;
    j.seq = seq;
    j.length = length;
    j.rads = rads;
    j.R = R;
    j.dist_cutoff = dist_cutoff;
    /* max_num_dyes of HMMFitter (fitters/hmm-fitter.cc:30-52) */
    unsigned dmax = 0;
    for (int c = 0; c < m->num_channels; c++) {
        unsigned n = 0;
        for (int i = 0; i < length; i++)
            if (seq[i] == c) n++;
        if (n > dmax) dmax = n;
    }
    j.dmax = dmax;
    j.logp = logp;
    j.partial = (wpo_fit_sums*)calloc(threads, sizeof(wpo_fit_sums));
    fit_arg* args = (fit_arg*)calloc(threads, sizeof(fit_arg));
    pthread_mutex_init(&j.lock, NULL);
    pthread_t* th = (pthread_t*)calloc(threads, sizeof(pthread_t));
    for (int i = 0; i < threads; i++) {
        args[i].j = &j;
        args[i].id = i;
        pthread_create(&th[i], NULL, fit_worker, &args[i]);
    }
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    pthread_mutex_destroy(&j.lock);
    for (int i = 0; i < threads; i++) {
        const wpo_fit_sums* p = &j.partial[i];
        sums->edman_num += p->edman_num;
        sums->edman_den += p->edman_den;
        for (int t = 0; t < WPO_MAX_TIMESTEPS; t++) {
            sums->detach_x[t] += p->detach_x[t];
            sums->detach_n[t] += p->detach_n[t];
        }
        sums->init_block_num += p->init_block_num;
        sums->init_block_den += p->init_block_den;
        sums->cyc_block_num += p->cyc_block_num;
        sums->cyc_block_den += p->cyc_block_den;
        for (int c = 0; c < WPO_MAX_CHANNELS; c++) {
            sums->bleach_num[c] += p->bleach_num[c];
            sums->bleach_den[c] += p->bleach_den[c];
            sums->dud_num[c] += p->dud_num[c];
            sums->dud_den[c] += p->dud_den[c];
            for (int n = 0; n < 16; n++) {
                sums->emis_w[c][n] += p->emis_w[c][n];
                sums->emis_x[c][n] += p->emis_x[c][n];
                sums->emis_xx[c][n] += p->emis_xx[c][n];
            }
        }
    }
    free(th);
    free(args);
    free(j.partial);
}

/* ------------------------------------------------------- kNN classifier */
/* NNClassifier (classifiers/nn-classifier.cc:59-215) over dye-tracks
 * counts [N][T][C] with sources (id, count, hits) in CSR form.
 *
 * Entry coordinates: KDTEntry::operator[] (nn-classifier.cc:59-74), the
 * adjusted mu of channel c given the counts of every channel at t; the
 * query is the radiometry itself (KDTQuery, :94-98).  Squared distances
 * follow LeafNode::consider (kd-tree/leaf-node.h:31-62): FP64, summed in
 * groups of four then singly.
 *
 * Selection (WPO_NN_KDTREE, the reference's).  KBest::insert
 * (kd-tree/k-best.h:26-42) keeps entries while the hits of all but the
 * farthest reach k, popping at most one entry per insertion, so the set it
 * ends with depends on the kd-tree's visiting order.  The tree is built as
 * make_node does (kd-tree/make-node.h:28-80: split on the first dimension
 * of largest range, at the element nth_element of max-min-nth.h:20-116
 * leaves at the middle, a leaf when either side would hold fewer than k
 * entries) over the entries in their input order, and searched as
 * InternalNode::search / LeafNode::search (internal-node.h:39-60,
 * leaf-node.h:31-62) with a max-heap on (squared distance, tree position):
 * KDTree keeps the entries in the permuted vector and the heap compares
 * their addresses on equal distances.
 *
 * Selection (WPO_NN_PREFIX): the order-independent set KBest holds when
 * entries arrive nearest first: the shortest prefix of the entries sorted by
 * (squared distance, index) whose hits reach k (all entries if they never
 * do).
 *
 * Scores: classify_helper (:137-163): weight exp(-d^2 / (2 sig^2)),
 * score[id] += weight * hits / count, total += weight * hits, entries taken
 * farthest first (the order KBest::fill returns them), sources in list order.
 * Top h: classify(radiometry, h) (:183-203) returns up to h ids in ascending
 * score; ids are ordered by (score, id) here, the reference's heap leaves
 * equal scores in an unspecified order. */
typedef struct {
    double d2;
    int idx;
} nn_cand;

static int nn_cand_cmp(const void* a, const void* b) {
    const nn_cand* x = (const nn_cand*)a;
    const nn_cand* y = (const nn_cand*)b;
    if (x->d2 < y->d2) return -1;
    if (x->d2 > y->d2) return 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

typedef struct {
    int id;
    double score;
} nn_score;

static int nn_score_cmp(const void* a, const void* b) {
    const nn_score* x = (const nn_score*)a;
    const nn_score* y = (const nn_score*)b;
    if (x->score < y->score) return -1;
    if (x->score > y->score) return 1;
    return (x->id > y->id) - (x->id < y->id);
}

static int int_cmp(const void* a, const void* b) {
    int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

void wpo_nn_coords(const wpo_model* m, int T, const int16_t* counts, int N, double* out) {
    int C = m->num_channels;
    for (long e = 0; e < N; e++)
        for (int t = 0; t < T; t++) {
            unsigned cts[WPO_MAX_CHANNELS];
            for (int c = 0; c < C; c++) cts[c] = (unsigned)counts[(e * T + t) * C + c];
            for (int c = 0; c < C; c++) out[(e * T + t) * C + c] = wpo_adjusted_mu(m, c, cts);
        }
}

/* ---- kd-tree (kd-tree/make-node.h, max-min-nth.h) over a permutation of
 * the entries: pos[i] is the input index of the entry at tree position i. */
typedef struct {
    const double* coords;
    int D;
    int32_t* pos;
} kd_arr;

static double kd_val(const kd_arr* a, long i, int s) { return a->coords[(long)a->pos[i] * a->D + s]; }

static void kd_swap(kd_arr* a, long i, long j) {
    int32_t t = a->pos[i];
    a->pos[i] = a->pos[j];
    a->pos[j] = t;
}

/* partition (max-min-nth.h:20-52): returns the final left cursor and counts
 * the values equal to the pivot's as the scans meet them. */
static long kd_partition(kd_arr* a, long begin, long end, int s, long pivot, int* num_eq) {
    *num_eq = 0;
    long l = begin, r = end - 1;
    double pv = kd_val(a, pivot, s);
    kd_swap(a, pivot, r);
    while (l < r) {
        while (l < r) {
            double lv = kd_val(a, l, s);
            if (lv == pv) (*num_eq)++;
            if (lv > pv) {
                kd_swap(a, l, r);
                r--;
                break;
            }
            l++;
        }
        while (l < r) {
            double rv = kd_val(a, r, s);
            if (rv == pv) (*num_eq)++;
            if (rv <= pv) {
                kd_swap(a, r, l);
                l++;
                break;
            }
            r--;
        }
    }
    return l;
}

/* partition_alternate (max-min-nth.h:54-78): pivot value at end - 1. */
static void kd_partition_alternate(kd_arr* a, long begin, long end, int s) {
    long l = begin, r = end - 1;
    double pv = kd_val(a, r, s);
    while (l < r) {
        while (l < r) {
            if (kd_val(a, l, s) >= pv) {
                kd_swap(a, l, r);
                r--;
                break;
            }
            l++;
        }
        while (l < r) {
            if (kd_val(a, r, s) < pv) {
                kd_swap(a, r, l);
                l++;
                break;
            }
            r--;
        }
    }
}

/* nth_element (max-min-nth.h:86-107). */
static long kd_nth_element(kd_arr* a, long begin, long end, int s, long nth) {
    int num_eq;
    long pivot = kd_partition(a, begin, end, s, nth, &num_eq);
    long right = pivot, left = pivot - num_eq;
    if (left <= nth && nth <= right) {
        if (nth - left > right - nth) return right + 1;
        kd_partition_alternate(a, begin, right + 1, s);
        return left;
    } else if (nth < left) {
        kd_partition_alternate(a, begin, right + 1, s);
        return kd_nth_element(a, begin, left, s, nth);
    }
    return kd_nth_element(a, right + 1, end, s, nth);
}

static int kd_new_node(wpo_kd_tree* t) {
    if (t->num_nodes == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 64;
        t->nodes = (wpo_kd_node*)realloc(t->nodes, sizeof(wpo_kd_node) * t->cap);
    }
    return t->num_nodes++;
}

/* make_node (make-node.h:28-80). */
static int kd_make_node(wpo_kd_tree* t, kd_arr* a, int k, long begin, long end) {
    const int D = a->D;
    double mins[64], maxes[64];
    for (int i = 0; i < D; i++) {
        mins[i] = DBL_MAX;
        maxes[i] = DBL_MIN;
    }
    for (long e = begin; e < end; e++)
        for (int i = 0; i < D; i++) {
            double v = kd_val(a, e, i);
            if (v < mins[i]) mins[i] = v;   /* std::min(mins[i], v) */
            if (maxes[i] < v) maxes[i] = v; /* std::max(maxes[i], v) */
        }
    double best = -1.0;
    int s = -1;
    for (int i = 0; i < D; i++) {
        double range = maxes[i] - mins[i];
        if (range > best) {
            best = range;
            s = i;
        }
    }
    long nth = kd_nth_element(a, begin, end, s, begin + (end - begin) / 2);
    int id = kd_new_node(t);
    if (nth - begin < k || end - nth < k) {
        wpo_kd_node* n = &t->nodes[id];
        memset(n, 0, sizeof(*n));
        n->leaf = 1;
        n->begin = (int)begin;
        n->end = (int)end;
        return id;
    }
    double max_left = DBL_MIN, min_right = DBL_MAX;
    for (long e = begin; e < nth; e++) {
        double v = kd_val(a, e, s);
        if (max_left < v) max_left = v;
    }
    for (long e = nth; e < end; e++) {
        double v = kd_val(a, e, s);
        if (v < min_right) min_right = v;
    }
    int left = kd_make_node(t, a, k, begin, nth);
    int right = kd_make_node(t, a, k, nth, end);
    wpo_kd_node* n = &t->nodes[id];
    memset(n, 0, sizeof(*n));
    n->s = s;
    n->left = left;
    n->right = right;
    n->max_left = max_left;
    n->min_right = min_right;
    n->split = (max_left + min_right) / 2;
    return id;
}

int wpo_kd_tree_build(const double* coords, int N, int D, int k, wpo_kd_tree* out) {
    memset(out, 0, sizeof(*out));
    if (D > 64) return -1;
    out->N = N;
    out->D = D;
    out->pos = (int32_t*)malloc(sizeof(int32_t) * (N > 0 ? N : 1));
    for (int i = 0; i < N; i++) out->pos[i] = i;
    if (N == 0) return 0;
    kd_arr a = {coords, D, out->pos};
    out->root = kd_make_node(out, &a, k, 0, N);
    return 0;
}

void wpo_kd_tree_free(wpo_kd_tree* t) {
    free(t->nodes);
    free(t->pos);
    memset(t, 0, sizeof(*t));
}

/* KBest (k-best.h:22-62): a max-heap on (squared distance, tree position),
 * the order of std::pair<double, E*>. */
typedef struct {
    double d;
    int pos;
} kb_item;

typedef struct {
    kb_item* heap;
    int n, cap;
    int k, hits;
    double kth;
    const int* pos_hits; /* hits of the entry at each tree position */
} kbest;

static int kb_less(kb_item a, kb_item b) { return a.d < b.d || (!(b.d < a.d) && a.pos < b.pos); }

static void kb_push(kbest* kb, kb_item it) {
    if (kb->n == kb->cap) {
        kb->cap = kb->cap ? 2 * kb->cap : 1024;
        kb->heap = (kb_item*)realloc(kb->heap, sizeof(kb_item) * kb->cap);
    }
    int i = kb->n++;
    while (i > 0) {
        int p = (i - 1) / 2;
        if (!kb_less(kb->heap[p], it)) break;
        kb->heap[i] = kb->heap[p];
        i = p;
    }
    kb->heap[i] = it;
}

static void kb_pop(kbest* kb) {
    kb_item last = kb->heap[--kb->n];
    int i = 0;
    for (;;) {
        int c = 2 * i + 1;
        if (c >= kb->n) break;
        if (c + 1 < kb->n && kb_less(kb->heap[c], kb->heap[c + 1])) c++;
        if (!kb_less(last, kb->heap[c])) break;
        kb->heap[i] = kb->heap[c];
        i = c;
    }
    if (kb->n > 0) kb->heap[i] = last;
}

/* KBest::insert (k-best.h:26-42). */
static void kb_insert(kbest* kb, double d, int pos) {
    kb->hits += kb->pos_hits[pos];
    kb_item it = {d, pos};
    kb_push(kb, it);
    int top_hits = kb->pos_hits[kb->heap[0].pos];
    if (kb->hits - top_hits >= kb->k) {
        kb->hits -= top_hits;
        kb_pop(kb);
    }
    if (kb->hits >= kb->k) kb->kth = kb->heap[0].d;
}

/* LeafNode::consider (leaf-node.h:31-62): FP64, groups of four with the
 * early exit, then singly. */
static void kd_consider(const wpo_kd_tree* t, const double* tree_coords, const double* q, int pos,
                        kbest* kb) {
    const int D = t->D;
    const double* x = tree_coords + (long)pos * D;
    double kth = kb->kth;
    double d2 = 0.0;
    int i = 0;
    while (i < D - 3) {
        double x1 = q[i] - x[i], x2 = q[i + 1] - x[i + 1];
        double x3 = q[i + 2] - x[i + 2], x4 = q[i + 3] - x[i + 3];
        d2 += x1 * x1 + x2 * x2 + x3 * x3 + x4 * x4;
        if (d2 >= kth) return;
        i += 4;
    }
    while (i < D) {
        double xx = q[i] - x[i];
        d2 += xx * xx;
        i++;
    }
    if (d2 >= kth) return;
    kb_insert(kb, d2, pos);
}

/* InternalNode::search / LeafNode::search (internal-node.h:39-60,
 * leaf-node.h:25-29). */
static void kd_search(const wpo_kd_tree* t, const double* tree_coords, int node, const double* q,
                      kbest* kb) {
    const wpo_kd_node* n = &t->nodes[node];
    if (n->leaf) {
        for (int p = n->begin; p < n->end; p++) kd_consider(t, tree_coords, q, p, kb);
        return;
    }
    double qv = q[n->s];
    if (qv < n->split) {
        kd_search(t, tree_coords, n->left, q, kb);
        double rd = n->min_right - qv;
        if (kb->kth > rd * rd) kd_search(t, tree_coords, n->right, q, kb);
    } else {
        kd_search(t, tree_coords, n->right, q, kb);
        double ld = qv - n->max_left;
        if (kb->kth > ld * ld) kd_search(t, tree_coords, n->left, q, kb);
    }
}

int wpo_kd_tree_search(const wpo_kd_tree* t, const double* tree_coords, const int* pos_hits,
                       const double* q, int k, int32_t* out_pos, double* out_d2, int max_out) {
    kbest kb;
    memset(&kb, 0, sizeof(kb));
    kb.k = k;
    kb.kth = DBL_MAX;
    kb.pos_hits = pos_hits;
    if (t->N > 0) kd_search(t, tree_coords, t->root, q, &kb);
    /* KBest::fill: farthest first */
    int n = 0;
    while (kb.n > 0) {
        if (n < max_out) {
            out_pos[n] = kb.heap[0].pos;
            out_d2[n] = kb.heap[0].d;
        }
        n++;
        kb_pop(&kb);
    }
    free(kb.heap);
    return n;
}

typedef struct {
    const double* coords;
    int N, D;
    int selection;
    /* WPO_NN_KDTREE: the tree, coordinates and hits in tree order */
    wpo_kd_tree tree;
    double* tree_coords;
    int* pos_hits;
    const int32_t *src_off, *src_id, *src_count, *src_hits;
    const int32_t* uniq; /* sorted distinct source ids */
    int U;
    const double* rads;
    int R, k, h;
    double two_sig_sq;
    int32_t* out_ncand;
    int32_t* out_cand_id;
    double* out_cand_score;
    double* out_total;
    /* hybrid (when seqs != NULL) */
    const wpo_model* m;
    int T;
    const int16_t* seqs;
    const int32_t* offsets;
    const int32_t* pep_ids;
    const int32_t* pep_counts;
    int P;
    unsigned dmax;
    double dist_cutoff;
    int32_t* hy_id;
    double* hy_score;
    double* hy_total;
    int next;
    pthread_mutex_t lock;
} nn_job;

/* HybridClassifier::classify (hybrid-classifier.cc:55-81) after the kNN
 * stage of read r: peptide indices of the candidates through the id map
 * (absent ids read as index 0 and count 0, unordered_map operator[]), the
 * HMM over them in ascending kNN score, the score times the subfraction,
 * the NaN patch. */
static void hybrid_one(const nn_job* j, int r) {
    int nc = j->out_ncand[r];
    if (nc == 0) {
        j->hy_id[r] = -1;
        j->hy_score[r] = 0.0;
        j->hy_total[r] = 1.0;
        return;
    }
    int32_t* cand = (int32_t*)malloc(sizeof(int32_t) * nc);
    double sub = 0.0;
    double total = j->out_total[r];
    for (int i = 0; i < nc; i++) {
        int id = j->out_cand_id[(long)r * j->h + i];
        int idx = 0, cnt = 0;
        for (int p = 0; p < j->P; p++) /* the map keeps the last peptide with an id */
            if (j->pep_ids[p] == id) {
                idx = p;
                cnt = j->pep_counts[p];
            }
        cand[i] = idx;
        sub += (j->out_cand_score[(long)r * j->h + i] / total) * (double)cnt;
    }
    int32_t id;
    double score, tot;
    classify_with_dmax(j->m, j->T, j->seqs, j->offsets, j->pep_ids, j->pep_counts, j->P, cand, nc,
                       j->rads + (long)r * j->D, j->dist_cutoff, j->dmax, &id, &score, &tot);
    free(cand);
    score *= sub;
    if (isnan(score / tot)) {
        score = 0.0;
        tot = 1.0;
    }
    j->hy_id[r] = id;
    j->hy_score[r] = score;
    j->hy_total[r] = tot;
}

static void nn_one(const nn_job* j, int r, nn_cand* cand, double* acc, nn_score* sc) {
    const double* q = j->rads + (long)r * j->D;
    const int D = j->D;
    long total_hits = 0;
    int m = 0;
    if (j->selection == WPO_NN_KDTREE) {
        /* KDTree::search then KBest::fill: farthest first; cand[] is kept
         * nearest first like the prefix path (reversed below). */
        int32_t* pos = (int32_t*)malloc(sizeof(int32_t) * (j->N > 0 ? j->N : 1));
        double* d2s = (double*)malloc(sizeof(double) * (j->N > 0 ? j->N : 1));
        m = wpo_kd_tree_search(&j->tree, j->tree_coords, j->pos_hits, q, j->k, pos, d2s, j->N);
        for (int i = 0; i < m; i++) {
            cand[m - 1 - i].d2 = d2s[i];
            cand[m - 1 - i].idx = j->tree.pos[pos[i]];
        }
        free(pos);
        free(d2s);
        goto scores;
    }
    for (int e = 0; e < j->N; e++) {
        const double* x = j->coords + (long)e * D;
        double d2 = 0.0;
        int i = 0;
        while (i < D - 3) {
            double x1 = q[i] - x[i], x2 = q[i + 1] - x[i + 1];
            double x3 = q[i + 2] - x[i + 2], x4 = q[i + 3] - x[i + 3];
            d2 += x1 * x1 + x2 * x2 + x3 * x3 + x4 * x4;
            i += 4;
        }
        while (i < D) {
            double xx = q[i] - x[i];
            d2 += xx * xx;
            i++;
        }
        cand[e].d2 = d2;
        cand[e].idx = e;
    }
    qsort(cand, j->N, sizeof(nn_cand), nn_cand_cmp);
    for (; m < j->N;) {
        int e = cand[m].idx;
        for (int s = j->src_off[e]; s < j->src_off[e + 1]; s++) total_hits += j->src_hits[s];
        m++;
        if (total_hits >= j->k) break;
    }
scores:
    for (int u = 0; u < j->U; u++) acc[u] = 0.0;
    double total = 0.0;
    for (int i = m - 1; i >= 0; i--) { /* farthest first */
        int e = cand[i].idx;
        double w = exp(-cand[i].d2 / j->two_sig_sq);
        for (int s = j->src_off[e]; s < j->src_off[e + 1]; s++) {
            const int32_t* p = (const int32_t*)bsearch(&j->src_id[s], j->uniq, j->U, sizeof(int32_t), int_cmp);
            int u = (int)(p - j->uniq);
            double hits = (double)j->src_hits[s], count = (double)j->src_count[s];
            total += w * hits;
            acc[u] += w * hits / count;
        }
    }
    int n = 0;
    for (int i = 0; i < m; i++) {
        int e = cand[i].idx;
        for (int s = j->src_off[e]; s < j->src_off[e + 1]; s++) {
            const int32_t* p = (const int32_t*)bsearch(&j->src_id[s], j->uniq, j->U, sizeof(int32_t), int_cmp);
            int u = (int)(p - j->uniq);
            if (acc[u] >= 0.0) { /* first visit: emit, then mark */
                sc[n].id = j->uniq[u];
                sc[n].score = acc[u];
                n++;
                acc[u] = -1.0 - acc[u];
            }
        }
    }
    qsort(sc, n, sizeof(nn_score), nn_score_cmp);
    int keep = n < j->h ? n : j->h;
    j->out_ncand[r] = keep;
    for (int i = 0; i < keep; i++) {
        j->out_cand_id[(long)r * j->h + i] = sc[n - keep + i].id;
        j->out_cand_score[(long)r * j->h + i] = sc[n - keep + i].score;
    }
    j->out_total[r] = total;
}

static void* nn_worker(void* arg) {
    nn_job* j = (nn_job*)arg;
    nn_cand* cand = (nn_cand*)malloc(sizeof(nn_cand) * (j->N > 0 ? j->N : 1));
    double* acc = (double*)malloc(sizeof(double) * (j->U > 0 ? j->U : 1));
    long ns = j->N > 0 ? j->src_off[j->N] : 0;
    nn_score* sc = (nn_score*)malloc(sizeof(nn_score) * (ns > 0 ? ns : 1));
    for (;;) {
        pthread_mutex_lock(&j->lock);
        int r = j->next++;
        pthread_mutex_unlock(&j->lock);
        if (r >= j->R) break;
        nn_one(j, r, cand, acc, sc);
        if (j->seqs) hybrid_one(j, r);
    }
    free(cand);
    free(acc);
    free(sc);
    return NULL;
}

static void nn_run_job(nn_job* j, const wpo_model* m, int T, const int16_t* track_counts, int N,
                       const int32_t* src_off, const int32_t* src_id, const int32_t* src_count,
                       const int32_t* src_hits, const double* rads, int R, int k, double sig, int h,
                       int threads) {
    if (threads < 1) threads = 1;
    int C = m->num_channels;
    j->D = T * C;
    j->N = N;
    double* coords = (double*)malloc(sizeof(double) * ((long)N * j->D + 1));
    wpo_nn_coords(m, T, track_counts, N, coords);
    j->coords = coords;
    j->src_off = src_off;
    j->src_id = src_id;
    j->src_count = src_count;
    j->src_hits = src_hits;
    long ns = N > 0 ? src_off[N] : 0;
    int32_t* uniq = (int32_t*)malloc(sizeof(int32_t) * (ns > 0 ? ns : 1));
    memcpy(uniq, src_id, sizeof(int32_t) * ns);
    qsort(uniq, ns, sizeof(int32_t), int_cmp);
    int U = 0;
    for (long i = 0; i < ns; i++)
        if (U == 0 || uniq[U - 1] != uniq[i]) uniq[U++] = uniq[i];
    j->uniq = uniq;
    j->U = U;
    j->rads = rads;
    j->R = R;
    j->k = k;
    j->h = h;
    j->two_sig_sq = 2.0 * sig * sig;
    if (j->selection == WPO_NN_KDTREE) {
        wpo_kd_tree_build(coords, N, j->D, k, &j->tree);
        j->tree_coords = (double*)malloc(sizeof(double) * ((long)N * j->D + 1));
        j->pos_hits = (int*)malloc(sizeof(int) * (N > 0 ? N : 1));
        for (long p = 0; p < N; p++) {
            int e = j->tree.pos[p];
            memcpy(j->tree_coords + p * j->D, coords + (long)e * j->D, sizeof(double) * j->D);
            int hits = 0;
            for (int s = src_off[e]; s < src_off[e + 1]; s++) hits += src_hits[s];
            j->pos_hits[p] = hits;
        }
    }
    pthread_mutex_init(&j->lock, NULL);
    pthread_t* th = (pthread_t*)calloc(threads, sizeof(pthread_t));
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, nn_worker, j);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    pthread_mutex_destroy(&j->lock);
    free(th);
    free(coords);
    free(uniq);
    if (j->selection == WPO_NN_KDTREE) {
        wpo_kd_tree_free(&j->tree);
        free(j->tree_coords);
        free(j->pos_hits);
    }
}

void wpo_nn_classify_batch(const wpo_model* m, int T, const int16_t* track_counts, int N,
                           const int32_t* src_off, const int32_t* src_id,
                           const int32_t* src_count, const int32_t* src_hits,
                           const double* rads, int R, int k, double sig, int h,
                           int selection, int threads, int32_t* out_ncand, int32_t* out_cand_id,
                           double* out_cand_score, double* out_total) {
    nn_job j;
    memset(&j, 0, sizeof(j));
    j.selection = selection;
    j.out_ncand = out_ncand;
    j.out_cand_id = out_cand_id;
    j.out_cand_score = out_cand_score;
    j.out_total = out_total;
    nn_run_job(&j, m, T, track_counts, N, src_off, src_id, src_count, src_hits, rads, R, k, sig, h,
               threads);
}

void wpo_hybrid_classify_batch(const wpo_model* m, int T, const int16_t* track_counts, int N,
                               const int32_t* src_off, const int32_t* src_id,
                               const int32_t* src_count, const int32_t* src_hits,
                               const int16_t* seqs, const int32_t* offsets, const int32_t* ids,
                               const int32_t* counts, int P, const double* rads, int R, int k,
                               double sig, int h, double dist_cutoff, int selection, int threads,
                               int32_t* out_id, double* out_score, double* out_total) {
    nn_job j;
    memset(&j, 0, sizeof(j));
    j.selection = selection;
    j.out_ncand = (int32_t*)malloc(sizeof(int32_t) * (R > 0 ? R : 1));
    j.out_cand_id = (int32_t*)malloc(sizeof(int32_t) * ((long)R * h + 1));
    j.out_cand_score = (double*)malloc(sizeof(double) * ((long)R * h + 1));
    j.out_total = (double*)malloc(sizeof(double) * (R > 0 ? R : 1));
    j.m = m;
    j.T = T;
    j.seqs = seqs;
    j.offsets = offsets;
    j.pep_ids = ids;
    j.pep_counts = counts;
    j.P = P;
    j.dmax = max_num_dyes_of(m->num_channels, seqs, offsets, P, T);
    j.dist_cutoff = dist_cutoff;
    j.hy_id = out_id;
    j.hy_score = out_score;
    j.hy_total = out_total;
    nn_run_job(&j, m, T, track_counts, N, src_off, src_id, src_count, src_hits, rads, R, k, sig, h,
               threads);
    free(j.out_ncand);
    free(j.out_cand_id);
    free(j.out_cand_score);
    free(j.out_total);
}

/* ---- dye-track dedup (simulation/dedup-dye-tracks.cc:35-141) ----------- */

typedef struct {
    const int16_t* counts;
    const int32_t* ids;
    int TC;
} dedup_ctx;

static dedup_ctx g_dedup;  /* qsort has no context argument in C11 */

static int dedup_cmp(const void* a, const void* b) {
    const int i = *(const int*)a, j = *(const int*)b;
    const int16_t* x = g_dedup.counts + (long)i * g_dedup.TC;
    const int16_t* y = g_dedup.counts + (long)j * g_dedup.TC;
    for (int k = 0; k < g_dedup.TC; k++)
        if (x[k] != y[k]) return x[k] < y[k] ? -1 : 1;
    if (g_dedup.ids[i] != g_dedup.ids[j]) return g_dedup.ids[i] < g_dedup.ids[j] ? -1 : 1;
    return i < j ? -1 : (i > j);  /* first instance of an id first */
}

int wpo_dedup_dye_tracks(int T, int C, int n, const int16_t* counts, const int32_t* ids,
                         const int32_t* cnts, int16_t* out_counts, int32_t* out_src_off,
                         int32_t* out_src_id, int32_t* out_src_count, int32_t* out_src_hits,
                         int32_t* out_num_sources) {
    const int TC = T * C;
    int* order = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
    for (int i = 0; i < n; i++) order[i] = i;
    g_dedup.counts = counts;
    g_dedup.ids = ids;
    g_dedup.TC = TC;
    qsort(order, n, sizeof(int), dedup_cmp);
    int u = 0, s = 0;
    out_src_off[0] = 0;
    for (int a = 0; a < n;) {
        /* one distinct track: the key of the reference's map-reduce */
        const int16_t* key = counts + (long)order[a] * TC;
        int b = a;
        while (b < n && memcmp(counts + (long)order[b] * TC, key, sizeof(int16_t) * TC) == 0) b++;
        memcpy(out_counts + (long)u * TC, key, sizeof(int16_t) * TC);
        /* reduce_dye_tracks_helper: one entry per source id */
        for (int i = a; i < b;) {
            int j = i;
            while (j < b && ids[order[j]] == ids[order[i]]) j++;
            out_src_id[s] = ids[order[i]];
            out_src_count[s] = cnts[order[i]];
            out_src_hits[s] = j - i;
            s++;
            i = j;
        }
        out_src_off[++u] = s;
        a = b;
    }
    free(order);
    *out_num_sources = s;
    return u;
}

/* ---- dye-track generation (simulation/generate-dye-track.cc:29-110) ---- */

typedef struct {
    uint64_t s[4];
} xoshiro;

static uint64_t splitmix64(uint64_t* x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* xoshiro256** (Blackman and Vigna) -> uniform double in [0, 1) */
static double xo_uniform(xoshiro* g) {
    uint64_t* s = g->s;
    const uint64_t r = rotl64(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return (double)(r >> 11) * 0x1.0p-53;
}

/* bernoulli_distribution(p)(gen) */
static int xo_bernoulli(xoshiro* g, double p) { return xo_uniform(g) < p; }

/* generate_dye_track for one dye-seq of length L: counts [T][C]. */
static void gen_dye_track(const wpo_model* m, const double* p_det, int T, const int16_t* seq, int L,
                          xoshiro* g, int16_t* ds, int16_t* out) {
    const int C = m->num_channels;
    memcpy(ds, seq, sizeof(int16_t) * L);
    for (int i = 0; i < L; i++)  /* duds */
        if (ds[i] != -1 && xo_bernoulli(g, m->p_dud[ds[i]])) ds[i] = -1;
    int16_t cnt[WPO_MAX_CHANNELS] = {0};
    for (int i = 0; i < L; i++)
        if (ds[i] != -1) cnt[ds[i]]++;
    int e = 0;
    int block = xo_bernoulli(g, m->p_initial_block);
    for (int t = 0; t < T; t++) {
        if (e < L) {
            for (int c = 0; c < C; c++) out[t * C + c] = cnt[c];
            if (xo_bernoulli(g, m->p_cyclic_block)) block = 1;
            if (xo_bernoulli(g, p_det[t])) {  /* detach */
                e = L;
                continue;
            }
            if (!block && !xo_bernoulli(g, m->p_edman_failure)) {
                if (ds[e] != -1) cnt[ds[e]]--;
                e++;
            }
            for (int i = e; i < L; i++)  /* bleaching */
                if (ds[i] != -1 && xo_bernoulli(g, m->p_bleach[ds[i]])) {
                    cnt[ds[i]]--;
                    ds[i] = -1;
                }
        } else {
            for (int c = 0; c < C; c++) out[t * C + c] = 0;
        }
    }
}

int wpo_simulate_dt(const wpo_model* m, int T, const int16_t* seqs, const int32_t* offsets,
                    const int32_t* ids, const int32_t* counts, int P, int per_peptide,
                    uint64_t seed, int16_t* out_counts, int32_t* out_src_off,
                    int32_t* out_src_id, int32_t* out_src_count, int32_t* out_src_hits,
                    int32_t* out_num_sources, int32_t* out_instances) {
    const int C = m->num_channels, TC = T * C;
    long n = 0;
    int Lmax = 1;
    for (int p = 0; p < P; p++) {
        n += (long)counts[p] * per_peptide;
        if (offsets[p + 1] - offsets[p] > Lmax) Lmax = offsets[p + 1] - offsets[p];
    }
    double p_det[WPO_MAX_TIMESTEPS];
    for (int t = 0; t < T; t++) p_det[t] = wpo_p_detach_at(m, (unsigned)t);
    xoshiro g;
    uint64_t sm = seed;
    for (int k = 0; k < 4; k++) g.s[k] = splitmix64(&sm);
    int16_t* tracks = (int16_t*)malloc(sizeof(int16_t) * (n > 0 ? n : 1) * TC);
    int32_t* tid = (int32_t*)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    int32_t* tcnt = (int32_t*)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    int16_t* ds = (int16_t*)malloc(sizeof(int16_t) * Lmax);
    long kept = 0;
    for (int p = 0; p < P; p++)
        for (long r = 0; r < (long)counts[p] * per_peptide; r++) {
            int16_t* tr = tracks + kept * TC;
            gen_dye_track(m, p_det, T, seqs + offsets[p], offsets[p + 1] - offsets[p], &g, ds, tr);
            int nontrivial = 0;
            for (int c = 0; c < C; c++) nontrivial |= tr[c] != 0;
            if (nontrivial) {
                tid[kept] = ids[p];
                tcnt[kept] = counts[p];
                kept++;
            }
        }
    const int u = wpo_dedup_dye_tracks(T, C, (int)kept, tracks, tid, tcnt, out_counts, out_src_off, out_src_id,
                                       out_src_count, out_src_hits, out_num_sources);
    *out_instances = (int32_t)kept;
    free(tracks);
    free(tid);
    free(tcnt);
    free(ds);
    return u;
}

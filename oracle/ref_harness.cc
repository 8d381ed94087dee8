// ref_harness.cc -- C entry points over the reference's own classes.
//
// TEST INFRASTRUCTURE ONLY.  Compiled (by oracle/Makefile) together with the
// reference's unmodified sources read in place from the reference checkout;
// the output goes to oracle/_ref/ and is never committed.  It drives the
// reference exactly the way its unit tests do (cc_code/src/hmm/hmm/
// peptide-hmm.test.cc:154-188) and the way its CLI does
// (cc_code/src/main/run-classify-hmm.cc:38-98, run-fit.cc:37-137), so that
// the CPU oracle (wp_oracle.c) and the CUDA path can be compared with the
// reference itself on the same inputs.
#include <omp.h>

#include <cmath>
#include <string>
#include <vector>

#include "classifiers/hmm-classifier.h"
#include "classifiers/hybrid-classifier.h"
#include "classifiers/nn-classifier.h"
#include "kd-tree/kd-tree.h"
#include "common/dye-track.h"
#include "common/dye-seq.h"
#include "common/radiometry.h"
#include "common/scored-classification.h"
#include "common/sourced-data.h"
#include "fitters/hmm-fitter.h"
#include "hmm/hmm/peptide-hmm.h"
#include "hmm/precomputations/dye-seq-precomputations.h"
#include "hmm/precomputations/radiometry-precomputations.h"
#include "hmm/precomputations/universal-precomputations.h"
#include "parameterization/fit/sequencing-model-fitter.h"
#include "parameterization/model/sequencing-model.h"
#include "parameterization/settings/fit-settings.h"
#include "parameterization/settings/sequencing-settings.h"
#include "simulation/dedup-dye-tracks.h"
#include "simulation/generate-dye-track.h"
#include "simulation/generate-dye-tracks.h"
#include "util/levmar-helper.h"
#include "wp_oracle.h"

using namespace whatprot;

namespace {

void to_reference(const wpo_model* m, SequencingModel* sm) {
    sm->p_edman_failure = m->p_edman_failure;
    sm->p_detach.base = m->p_detach;
    sm->p_detach.initial = m->p_initial_detach;
    sm->p_detach.initial_decay = m->p_initial_detach_decay;
    sm->p_initial_block = m->p_initial_block;
    sm->p_cyclic_block = m->p_cyclic_block;
    int C = m->num_channels;
    for (int c = 0; c < C; c++) {
        ChannelModel* cm = new ChannelModel(c, C);
        cm->p_bleach = m->p_bleach[c];
        cm->p_dud = m->p_dud[c];
        cm->bg_sig = m->bg_sig[c];
        cm->mu = m->mu[c];
        cm->sig = m->sig[c];
        for (int o = 0; o < C; o++) {
            cm->interactions[o] = m->interactions[c][o];
            cm->flat_interactions[o] = m->flat_interactions[c][o];
        }
        sm->channel_models.push_back(cm);
    }
}

void from_reference(const SequencingModel& sm, int C, wpo_model* m) {
    m->num_channels = C;
    m->p_edman_failure = sm.p_edman_failure;
    m->p_detach = sm.p_detach.base;
    m->p_initial_detach = sm.p_detach.initial;
    m->p_initial_detach_decay = sm.p_detach.initial_decay;
    m->p_initial_block = sm.p_initial_block;
    m->p_cyclic_block = sm.p_cyclic_block;
    for (int c = 0; c < C; c++) {
        m->p_bleach[c] = sm.channel_models[c]->p_bleach;
        m->p_dud[c] = sm.channel_models[c]->p_dud;
        m->bg_sig[c] = sm.channel_models[c]->bg_sig;
        m->mu[c] = sm.channel_models[c]->mu;
        m->sig[c] = sm.channel_models[c]->sig;
    }
}

Radiometry make_radiometry(int T, int C, const double* rad) {
    Radiometry r(T, C);
    for (int t = 0; t < T; t++)
        for (int c = 0; c < C; c++) r(t, c) = rad[t * C + c];
    return r;
}

typedef SourcedData<DyeTrack, SourceCountHitsList<int>> TrackData;

// Dye-tracks [N][T][C] with CSR sources as the reference's deduplicated
// training set (dedup-dye-tracks.cc:118-141).
std::vector<TrackData> make_tracks(int T, int C, const int16_t* counts, int N,
                                   const int32_t* src_off, const int32_t* src_id,
                                   const int32_t* src_count, const int32_t* src_hits) {
    std::vector<TrackData> out;
    out.reserve(N);
    std::vector<short> buf(T * C);
    for (int e = 0; e < N; e++) {
        for (int i = 0; i < T * C; i++) buf[i] = counts[(long)e * T * C + i];
        int ns = src_off[e + 1] - src_off[e];
        SourceCountHits<int>** srcs = new SourceCountHits<int>*[ns];
        for (int j = 0; j < ns; j++) {
            int s = src_off[e] + j;
            srcs[j] = new SourceCountHits<int>(src_id[s], src_count[s], src_hits[s]);
        }
        out.push_back(TrackData(DyeTrack(T, C, buf.data()), SourceCountHitsList<int>(ns, srcs)));
    }
    return out;
}

// An entry for the reference's KDTree template that remembers its input
// index (the template's requirements, kd-tree/kd-tree.h:22-31).
struct OrderEntry {
    std::vector<double> x;
    int index = 0;
    int hits = 1;
    double operator[](int i) const { return x[i]; }
};

}  // namespace

extern "C" {

// KDTree's constructor (kd-tree/kd-tree.h:36-43) over coords [N][D] for k:
// the input index of the entry at each position of its permuted vector.
void ref_kd_tree_order(const double* coords, int N, int D, int k, int32_t* perm) {
    std::vector<OrderEntry> v(N);
    for (int i = 0; i < N; i++) {
        v[i].x.assign(coords + (long)i * D, coords + (long)(i + 1) * D);
        v[i].index = i;
    }
    KDTree<OrderEntry, OrderEntry> tree(k, D, std::move(v));
    for (int i = 0; i < N; i++) perm[i] = tree.values[i].index;
}

// NNClassifier (nn-classifier.cc:100-215): for every read, classify(rad, h)
// into [R][h] (ascending score, *ncand entries) and classify(rad) into
// best_*; OpenMP over reads.
void ref_nn_classify(const wpo_model* m, int T, const int16_t* counts, int N,
                     const int32_t* src_off, const int32_t* src_id,
                     const int32_t* src_count, const int32_t* src_hits,
                     int R, const double* rads, int k, double sig, int h, int threads,
                     int32_t* out_ncand, int32_t* out_cand_id, double* out_cand_score,
                     double* out_cand_total, int32_t* out_best_id, double* out_best_score,
                     double* out_best_total, double* seconds) {
    int C = m->num_channels;
    SequencingModel sm;
    to_reference(m, &sm);
    std::vector<TrackData> tracks = make_tracks(T, C, counts, N, src_off, src_id, src_count, src_hits);
    NNClassifier nn(T, C, sm, k, sig, &tracks);
    if (threads > 0) omp_set_num_threads(threads);
    double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 1)
    for (int r = 0; r < R; r++) {
        Radiometry rad = make_radiometry(T, C, rads + (long)r * T * C);
        std::vector<ScoredClassification> top = nn.classify(rad, (unsigned)h);
        out_ncand[r] = (int)top.size();
        for (size_t i = 0; i < top.size(); i++) {
            out_cand_id[(long)r * h + i] = top[i].id;
            out_cand_score[(long)r * h + i] = top[i].score;
        }
        out_cand_total[r] = top.empty() ? 0.0 : top[0].total;
        ScoredClassification best = nn.classify(rad);
        out_best_id[r] = best.id;
        out_best_score[r] = best.score;
        out_best_total[r] = best.total;
    }
    double t1 = omp_get_wtime();
    if (seconds) *seconds = t1 - t0;
}

// HybridClassifier::classify(vector<Radiometry>) (hybrid-classifier.cc:
// 55-94), OpenMP over reads as the CLI runs it.
void ref_hybrid_classify(const wpo_model* m, int T, const int16_t* counts, int N,
                         const int32_t* src_off, const int32_t* src_id,
                         const int32_t* src_count, const int32_t* src_hits, int P,
                         const char* const* seqs, const int* ids, const int* pcounts, int R,
                         const double* rads, int k, double sig, int h, double dist_cutoff,
                         int threads, int* out_id, double* out_score, double* out_total,
                         double* seconds) {
    int C = m->num_channels;
    SequencingModel sm;
    to_reference(m, &sm);
    SequencingSettings ss;
    ss.dist_cutoff = dist_cutoff;
    std::vector<SourcedData<DyeSeq, SourceCount<int>>> dye_seqs;
    dye_seqs.reserve(P);
    for (int i = 0; i < P; i++)
        dye_seqs.push_back(SourcedData<DyeSeq, SourceCount<int>>(
                DyeSeq(C, std::string(seqs[i])), SourceCount<int>(ids[i], pcounts[i])));
    std::vector<TrackData> tracks = make_tracks(T, C, counts, N, src_off, src_id, src_count, src_hits);
    std::vector<Radiometry> radiometries;
    radiometries.reserve(R);
    for (int r = 0; r < R; r++)
        radiometries.push_back(make_radiometry(T, C, rads + (long)r * T * C));
    if (threads > 0) omp_set_num_threads(threads);
    HybridClassifier hybrid(T, C, sm, ss, k, sig, &tracks, h, dye_seqs);
    double t0 = omp_get_wtime();
    std::vector<ScoredClassification> results = hybrid.classify(radiometries);
    double t1 = omp_get_wtime();
    if (seconds) *seconds = t1 - t0;
    for (int r = 0; r < R; r++) {
        out_id[r] = results[r].id;
        out_score[r] = results[r].score;
        out_total[r] = results[r].total;
    }
}


// PeptideHMM(...).probability() for one pair, built as in
// peptide-hmm.test.cc:154-188.
double ref_peptide_probability(const wpo_model* m, int T, const char* dye_seq,
                               const double* rad, unsigned max_num_dyes,
                               double dist_cutoff) {
    int C = m->num_channels;
    SequencingModel sm;
    to_reference(m, &sm);
    SequencingSettings ss;
    ss.dist_cutoff = dist_cutoff;
    UniversalPrecomputations up(sm, T, C);
    up.set_max_num_dyes(max_num_dyes);
    DyeSeq ds(C, std::string(dye_seq));
    DyeSeqPrecomputations dsp(ds, sm, T, C);
    Radiometry r = make_radiometry(T, C, rad);
    RadiometryPrecomputations rp(r, sm, ss, max_num_dyes);
    PeptideHMM hmm(T, C, dsp, rp, up);
    return hmm.probability();
}

// HMMClassifier::classify(vector<Radiometry>) (hmm-classifier.cc:84-93),
// OpenMP-parallel over reads exactly as the CLI runs it.  *seconds receives
// the wall time of the classify call alone (run-classify-hmm.cc:85-88).
void ref_classify(const wpo_model* m, int T, int P, const char* const* seqs,
                  const int* ids, const int* counts, int R, const double* rads,
                  double dist_cutoff, int threads, int* out_id,
                  double* out_score, double* out_total, double* seconds) {
    int C = m->num_channels;
    SequencingModel sm;
    to_reference(m, &sm);
    SequencingSettings ss;
    ss.dist_cutoff = dist_cutoff;
    std::vector<SourcedData<DyeSeq, SourceCount<int>>> dye_seqs;
    dye_seqs.reserve(P);
    for (int i = 0; i < P; i++)
        dye_seqs.push_back(SourcedData<DyeSeq, SourceCount<int>>(
                DyeSeq(C, std::string(seqs[i])), SourceCount<int>(ids[i], counts[i])));
    std::vector<Radiometry> radiometries;
    radiometries.reserve(R);
    for (int r = 0; r < R; r++)
        radiometries.push_back(make_radiometry(T, C, rads + (long)r * T * C));
    if (threads > 0) omp_set_num_threads(threads);
    HMMClassifier classifier(T, C, sm, ss, dye_seqs);
    double t0 = omp_get_wtime();
    std::vector<ScoredClassification> results = classifier.classify(radiometries);
    double t1 = omp_get_wtime();
    if (seconds) *seconds = t1 - t0;
    for (int r = 0; r < R; r++) {
        out_id[r] = results[r].id;
        out_score[r] = results[r].score;
        out_total[r] = results[r].total;
    }
}

// GenericHMM::improve_fit for one read (generic-hmm.h:60-109) into a fresh
// SequencingModelFitter; returns P and the expected counts.
double ref_improve_fit(const wpo_model* m, int T, const char* dye_seq,
                       const double* rad, unsigned max_num_dyes,
                       double dist_cutoff, wpo_fit_sums* sums) {
    int C = m->num_channels;
    SequencingModel sm;
    to_reference(m, &sm);
    SequencingSettings ss;
    ss.dist_cutoff = dist_cutoff;
    UniversalPrecomputations up(sm, T, C);
    up.set_max_num_dyes(max_num_dyes);
    DyeSeq ds(C, std::string(dye_seq));
    DyeSeqPrecomputations dsp(ds, sm, T, C);
    Radiometry r = make_radiometry(T, C, rad);
    RadiometryPrecomputations rp(r, sm, ss, max_num_dyes);
    PeptideHMM hmm(T, C, dsp, rp, up);
    FitSettings fs(C);
    SequencingModelFitter smf(T, C, sm, fs);
    double p = hmm.improve_fit(&smf);
    sums->edman_num = smf.p_edman_failure_fit.numerator;
    sums->edman_den = smf.p_edman_failure_fit.denominator;
    for (int t = 0; t < T - 1; t++) {
        sums->detach_x[t] = smf.p_detach_fit.xvec[t];
        sums->detach_n[t] = smf.p_detach_fit.nvec[t];
    }
    sums->init_block_num = smf.p_initial_block_fit.numerator;
    sums->init_block_den = smf.p_initial_block_fit.denominator;
    sums->cyc_block_num = smf.p_cyclic_block_fit.numerator;
    sums->cyc_block_den = smf.p_cyclic_block_fit.denominator;
    for (int c = 0; c < C; c++) {
        sums->bleach_num[c] = smf.channel_fits[c]->p_bleach_fit.numerator;
        sums->bleach_den[c] = smf.channel_fits[c]->p_bleach_fit.denominator;
        sums->dud_num[c] = smf.channel_fits[c]->p_dud_fit.numerator;
        sums->dud_den[c] = smf.channel_fits[c]->p_dud_fit.denominator;
    }
    return p;
}

// One E-step of HMMFitter::fit (hmm-fitter.h:58-78) over R reads, the
// reads split across OpenMP threads (the reference runs them serially),
// each thread with its own SequencingModelFitter, added at the end.
// Returns the sum of the edman denominators (a checksum).
double ref_improve_fit_batch(const wpo_model* m, int T, const char* dye_seq,
                             int R, const double* rads, int threads) {
    int C = m->num_channels;
    SequencingModel sm;
    to_reference(m, &sm);
    SequencingSettings ss;
    ss.dist_cutoff = std::numeric_limits<double>::max();
    DyeSeq ds(C, std::string(dye_seq));
    unsigned max_num_dyes = 0;
    for (int c = 0; c < C; c++) {
        unsigned n = 0;
        for (unsigned i = 0; i < ds.length; i++)
            if (ds[i] == c) n++;
        if (n > max_num_dyes) max_num_dyes = n;
    }
    UniversalPrecomputations up(sm, T, C);
    up.set_max_num_dyes(max_num_dyes);
    DyeSeqPrecomputations dsp(ds, sm, T, C);
    FitSettings fs(C);
    double total = 0.0;
#pragma omp parallel num_threads(threads) reduction(+ : total)
    {
        SequencingModelFitter fitter(T, C, sm, fs);
#pragma omp for schedule(dynamic, 4)
        for (int r = 0; r < R; r++) {
            Radiometry rad = make_radiometry(T, C, rads + (long)r * T * C);
            RadiometryPrecomputations rp(rad, sm, ss, max_num_dyes);
            PeptideHMM hmm(T, C, dsp, rp, up);
            SequencingModelFitter pf(T, C, sm, fs);
            hmm.improve_fit(&pf);
            fitter += pf;
        }
        total += fitter.p_edman_failure_fit.denominator;
    }
    return total;
}

// HMMFitter::fit (hmm-fitter.h:49-116) with no holds and no pruning, as the
// `fit` CLI runs it (run-fit.cc:55-95).  Returns log(L) of the fitted model.
double ref_fit(const wpo_model* start, int T, const char* dye_seq, int R,
               const double* rads, double stopping_threshold,
               double max_runtime, wpo_model* out, double* step_size,
               double* seconds) {
    int C = start->num_channels;
    SequencingModel sm;
    to_reference(start, &sm);
    SequencingSettings ss;
    ss.dist_cutoff = std::numeric_limits<double>::max();
    FitSettings fs(C);
    DyeSeq ds(C, std::string(dye_seq));
    std::vector<Radiometry> radiometries;
    radiometries.reserve(R);
    for (int r = 0; r < R; r++)
        radiometries.push_back(make_radiometry(T, C, rads + (long)r * T * C));
    HMMFitter fitter(T, C, stopping_threshold, max_runtime, sm, ss, fs, ds);
    SequencingModel fitted;
    double t0 = omp_get_wtime();
    double log_l = fitter.fit(radiometries, &fitted, step_size);
    double t1 = omp_get_wtime();
    if (seconds) *seconds = t1 - t0;
    from_reference(fitted, C, out);
    for (int c = 0; c < C; c++)
        for (int o = 0; o < C; o++) {
            out->interactions[c][o] = start->interactions[c][o];
            out->flat_interactions[c][o] = start->flat_interactions[c][o];
        }
    return log_l;
}

/* least_squares_fit_of_offset_exponential (util/levmar-helper.cc:44-85)
 * on y, w (n points) from params[3], holds as non-zero held[k]. */
void ref_offset_exponential(const double* y, const double* w, int n,
                            const int* held, double* params) {
    std::vector<double> yv(y, y + n), wv(w, w + n), p(params, params + 3);
    std::vector<bool> hold(3);
    for (int k = 0; k < 3; k++) hold[k] = held[k] != 0;
    least_squares_fit_of_offset_exponential(yv, wv, hold, &p);
    for (int k = 0; k < 3; k++) params[k] = p[k];
}

// generate_dye_track (simulation/generate-dye-track.cc:29-110) n times for
// one dye-seq from std::default_random_engine(seed): counts [n][T][C].
void ref_generate_dye_tracks(const wpo_model* m, int T, const char* dye_seq, int n, unsigned seed,
                             int16_t* out) {
    int C = m->num_channels;
    SequencingModel sm;
    to_reference(m, &sm);
    DyeSeq ds(C, std::string(dye_seq));
    std::default_random_engine gen(seed);
    for (int i = 0; i < n; i++) {
        DyeTrack dt(T, C);
        generate_dye_track(sm, ds, T, C, &gen, &dt);
        for (int t = 0; t < T; t++)
            for (int c = 0; c < C; c++) out[((long)i * T + t) * C + c] = dt(t, c);
    }
}

// dedup_dye_tracks (simulation/dedup-dye-tracks.cc:35-61, on the vendored
// MapReduce-MPI with its serial stubs) over n given dye-tracks [n][T][C]
// with sources (ids[i], cnts[i]), as run-simulate-dt.cc:63-78 calls it.
// Writes the unique tracks, in the order the reference produces them, with
// CSR sources; the out arrays hold at least n tracks and n sources.
void ref_dedup_dye_tracks(int T, int C, int n, const int16_t* counts, const int* ids, const int* cnts,
                          int* out_num_tracks, int* out_num_sources, int16_t* out_counts, int* out_src_off,
                          int* out_src_id, int* out_src_count, int* out_src_hits) {
    std::vector<SourcedData<DyeTrack, SourceCount<int>>> in;
    in.reserve(n);
    for (int i = 0; i < n; i++) {
        DyeTrack dt(T, C);
        for (int t = 0; t < T; t++)
            for (int c = 0; c < C; c++) dt(t, c) = counts[((long)i * T + t) * C + c];
        in.push_back(SourcedData<DyeTrack, SourceCount<int>>(std::move(dt), SourceCount<int>(ids[i], cnts[i])));
    }
    std::vector<SourcedData<DyeTrack, SourceCountHitsList<int>>> out;
    dedup_dye_tracks(T, C, &in, &out);
    int s = 0;
    out_src_off[0] = 0;
    for (size_t u = 0; u < out.size(); u++) {
        for (int t = 0; t < T; t++)
            for (int c = 0; c < C; c++) out_counts[((long)u * T + t) * C + c] = out[u].value(t, c);
        for (int k = 0; k < out[u].source.num_sources; k++, s++) {
            out_src_id[s] = out[u].source.sources[k]->source;
            out_src_count[s] = out[u].source.sources[k]->count;
            out_src_hits[s] = out[u].source.sources[k]->hits;
        }
        out_src_off[u + 1] = s;
    }
    *out_num_tracks = (int)out.size();
    *out_num_sources = s;
}

// `simulate dt` (main/run-simulate-dt.cc:61-81): generate_dye_tracks over P
// dye-seqs with (ids, counts), per_peptide tracks per peptide copy, from
// std::default_random_engine(seed), then dedup_dye_tracks.  Returns the
// wall seconds of the two calls; writes the numbers of kept instances,
// distinct tracks and sources.
double ref_simulate_dt(const wpo_model* m, int T, int P, const char* const* seqs, const int* ids,
                       const int* counts, int per_peptide, unsigned seed, int* out_instances,
                       int* out_num_tracks, int* out_num_sources) {
    int C = m->num_channels;
    SequencingModel sm;
    to_reference(m, &sm);
    std::vector<SourcedData<DyeSeq, SourceCount<int>>> dye_seqs;
    for (int i = 0; i < P; i++)
        dye_seqs.push_back(SourcedData<DyeSeq, SourceCount<int>>(DyeSeq(C, std::string(seqs[i])),
                                                                 SourceCount<int>(ids[i], counts[i])));
    std::default_random_engine gen(seed);
    double t0 = omp_get_wtime();
    std::vector<SourcedData<DyeTrack, SourceCount<int>>> tracks;
    generate_dye_tracks(sm, dye_seqs, T, C, per_peptide, &gen, &tracks);
    std::vector<SourcedData<DyeTrack, SourceCountHitsList<int>>> out;
    dedup_dye_tracks(T, C, &tracks, &out);
    double t1 = omp_get_wtime();
    int s = 0;
    for (auto& d : out) s += d.source.num_sources;
    *out_instances = (int)tracks.size();
    *out_num_tracks = (int)out.size();
    *out_num_sources = s;
    return t1 - t0;
}

}  // extern "C"

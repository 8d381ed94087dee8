// whatprot_gpu.cc -- the classes of whatprot_gpu.h over the C ABI.
//
// Every conversion here is a copy of the caller's whatprot objects into the
// flat arrays the C ABI takes: the SequencingModel into wp_seq_model, the
// dye-seqs into one ragged int16 array (ids and counts beside it), the
// dye-tracks into [N][T][C] counts plus ragged sources, the radiometries
// into [R][T][C] doubles.  Results come back as ScoredClassification.
#include "whatprot_gpu.h"

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>

#include "../../include/whatprot_gb300.h"

namespace whatprot {
namespace gpu {

Context::Context() : ctx_(nullptr) {
    int device = 0;
    if (const char* s = std::getenv("WHATPROT_GPU_DEVICE")) device = std::atoi(s);
    const int st = wp_ctx_create(&ctx_, device);
    if (st != WP_OK || !ctx_)
        throw std::runtime_error("whatprot_gpu: no context on device " + std::to_string(device) + " (status " +
                                 std::to_string(st) + ")");
}

Context::~Context() {
    if (ctx_) wp_ctx_destroy(ctx_);
}

void Context::check(int st, const char* what) const {
    if (st != WP_OK)
        throw std::runtime_error(std::string("whatprot_gpu: ") + what + " failed (status " + std::to_string(st) +
                                 "): " + wp_last_error(ctx_));
}

namespace {

const Radiometry& deref(const Radiometry& r) { return r; }
const Radiometry& deref(const Radiometry* r) { return *r; }

template <class V>
std::vector<double> flatten_any(const V& radiometries) {
    std::vector<double> out;
    if (radiometries.empty()) return out;
    const Radiometry& first = deref(radiometries[0]);
    const size_t n = (size_t)first.num_timesteps * first.num_channels;
    out.resize(n * radiometries.size());
    for (size_t r = 0; r < radiometries.size(); r++) {
        const Radiometry& rad = deref(radiometries[r]);
        if ((size_t)rad.num_timesteps * rad.num_channels != n)
            throw std::invalid_argument("whatprot_gpu: radiometries of different shapes");
        for (size_t i = 0; i < n; i++) out[r * n + i] = rad.intensities[i];
    }
    return out;
}

// A SequencingModel as the C ABI's wp_seq_model; the per-channel arrays
// live in this object.
struct ModelArrays {
    std::vector<double> p_bleach, p_dud, bg_sig, mu, sig, inter, flat;
    wp_seq_model m;

    explicit ModelArrays(const SequencingModel& sm) {
        const int C = (int)sm.channel_models.size();
        for (int c = 0; c < C; c++) {
            const ChannelModel& cm = *sm.channel_models[c];
            p_bleach.push_back(cm.p_bleach);
            p_dud.push_back(cm.p_dud);
            bg_sig.push_back(cm.bg_sig);
            mu.push_back(cm.mu);
            sig.push_back(cm.sig);
            for (int o = 0; o < C; o++) {
                inter.push_back(o < (int)cm.interactions.size() ? cm.interactions[o] : 1.0);
                flat.push_back(o < (int)cm.flat_interactions.size() ? cm.flat_interactions[o] : 1.0);
            }
        }
        m.num_channels = C;
        m.p_edman_failure = sm.p_edman_failure;
        m.p_detach = sm.p_detach.base;
        m.p_initial_detach = sm.p_detach.initial;
        m.p_initial_detach_decay = sm.p_detach.initial_decay;
        m.p_initial_block = sm.p_initial_block;
        m.p_cyclic_block = sm.p_cyclic_block;
        m.p_bleach = p_bleach.data();
        m.p_dud = p_dud.data();
        m.bg_sig = bg_sig.data();
        m.mu = mu.data();
        m.sig = sig.data();
        m.interactions = inter.data();
        m.flat_interactions = flat.data();
    }
};

// The classifier's NaN patch (classifiers/hmm-classifier.h:73-76).
ScoredClassification patched(int id, double score, double total) {
    ScoredClassification r(id, score, total);
    if (std::isnan(r.adjusted_score())) {
        r.score = 0.0;
        r.total = 1.0;
    }
    return r;
}

std::vector<int16_t> dye_seq_array(const DyeSeq& d) {
    std::vector<int16_t> s(d.length);
    for (unsigned int i = 0; i < d.length; i++) s[i] = (int16_t)d.seq[i];
    return s;
}

}  // namespace

std::vector<double> flatten(const std::vector<Radiometry>& radiometries) { return flatten_any(radiometries); }
std::vector<double> flatten(const std::vector<Radiometry*>& radiometries) { return flatten_any(radiometries); }
std::vector<double> flatten(const std::vector<const Radiometry*>& radiometries) {
    return flatten_any(radiometries);
}

void upload_model(const Context& ctx, const SequencingModel& seq_model, unsigned int num_timesteps) {
    ModelArrays ma(seq_model);
    ctx.check(wp_model_upload(ctx.get(), &ma.m, (int)num_timesteps), "wp_model_upload");
}

void upload_dye_seqs(const Context& ctx, const std::vector<SourcedData<DyeSeq, SourceCount<int>>>& dye_seqs) {
    std::vector<int16_t> flat;
    std::vector<int32_t> off(1, 0), ids, counts;
    for (const auto& d : dye_seqs) {
        for (unsigned int i = 0; i < d.value.length; i++) flat.push_back((int16_t)d.value.seq[i]);
        off.push_back((int32_t)flat.size());
        ids.push_back(d.source.source);
        counts.push_back(d.source.count);
    }
    if (flat.empty()) flat.push_back(-1);  // a valid pointer for all-empty sequences
    ctx.check(wp_peptides_upload(ctx.get(), flat.data(), off.data(), ids.data(), counts.data(), (int)dye_seqs.size()),
              "wp_peptides_upload");
}

void upload_dye_tracks(const Context& ctx, unsigned int num_timesteps, unsigned int num_channels,
                       const std::vector<SourcedData<DyeTrack, SourceCountHitsList<int>>>& dye_tracks) {
    const size_t n = (size_t)num_timesteps * num_channels;
    std::vector<int16_t> counts;
    counts.reserve(n * dye_tracks.size());
    std::vector<int32_t> off(1, 0), sid, scnt, shit;
    for (const auto& dt : dye_tracks) {
        if (dt.value.counts.size() != n) throw std::invalid_argument("whatprot_gpu: dye-track of another shape");
        for (size_t i = 0; i < n; i++) counts.push_back((int16_t)dt.value.counts[i]);
        for (int j = 0; j < dt.source.num_sources; j++) {
            sid.push_back(dt.source.sources[j]->source);
            scnt.push_back(dt.source.sources[j]->count);
            shit.push_back(dt.source.sources[j]->hits);
        }
        off.push_back((int32_t)sid.size());
    }
    ctx.check(wp_nn_tracks_upload(ctx.get(), counts.data(), (int)dye_tracks.size(), (int)num_timesteps,
                                  (int)num_channels, off.data(), sid.data(), scnt.data(), shit.data()),
              "wp_nn_tracks_upload");
}

}  // namespace gpu

// ---------------------------------------------------------------- HMMClassifier

HMMClassifier::HMMClassifier(unsigned int num_timesteps,
                             unsigned int num_channels,
                             const SequencingModel& seq_model,
                             const SequencingSettings& seq_settings,
                             const std::vector<SourcedData<DyeSeq, SourceCount<int>>>& dye_seqs)
        : seq_model(seq_model),
          seq_settings(seq_settings),
          dye_seqs(dye_seqs),
          num_timesteps(num_timesteps),
          num_channels(num_channels),
          max_num_dyes(0) {
    for (const auto& d : dye_seqs) {
        unsigned int n = 0;
        for (unsigned int i = 0; i < d.value.length; i++) n += d.value.seq[i] >= 0 ? 1u : 0u;
        if (n > max_num_dyes) max_num_dyes = n;
    }
    gpu::upload_model(ctx, seq_model, num_timesteps);
    gpu::upload_dye_seqs(ctx, dye_seqs);
}

HMMClassifier::~HMMClassifier() {}

std::vector<ScoredClassification> HMMClassifier::run(const double* rads, int num_reads, const int* cand,
                                                     const int* cand_off) {
    std::vector<int32_t> id(num_reads);
    std::vector<double> score(num_reads), total(num_reads);
    if (num_reads > 0)
        ctx.check(wp_hmm_classify(ctx.get(), rads, num_reads, seq_settings.dist_cutoff, cand, cand_off, id.data(),
                                  score.data(), total.data(), nullptr),
                  "wp_hmm_classify");
    std::vector<ScoredClassification> out;
    out.reserve(num_reads);
    for (int r = 0; r < num_reads; r++) out.push_back(ScoredClassification(id[r], score[r], total[r]));
    return out;
}

ScoredClassification HMMClassifier::classify(const Radiometry& radiometry) {
    return run(radiometry.intensities, 1, nullptr, nullptr)[0];
}

ScoredClassification HMMClassifier::classify(const Radiometry& radiometry, const std::vector<int>& candidate_indices) {
    std::vector<int32_t> cand(candidate_indices.begin(), candidate_indices.end());
    for (int32_t c : cand)
        if (c < 0 || c >= (int32_t)dye_seqs.size()) throw std::out_of_range("whatprot_gpu: candidate index");
    const int32_t off[2] = {0, (int32_t)cand.size()};
    if (cand.empty()) cand.push_back(0);
    return run(radiometry.intensities, 1, cand.data(), off)[0];
}

std::vector<ScoredClassification> HMMClassifier::classify(const std::vector<Radiometry>& radiometries) {
    const std::vector<double> rads = gpu::flatten(radiometries);
    return run(rads.data(), (int)radiometries.size(), nullptr, nullptr);
}

// ---------------------------------------------------------------- NNClassifier

NNClassifier::NNClassifier(unsigned int num_timesteps,
                           unsigned int num_channels,
                           const SequencingModel& seq_model,
                           int k,
                           double sig,
                           std::vector<SourcedData<DyeTrack, SourceCountHitsList<int>>>* dye_tracks)
        : num_train((int)dye_tracks->size()),
          num_timesteps(num_timesteps),
          num_channels(num_channels),
          k(k),
          two_sig_sq(2.0 * sig * sig),
          sig(sig) {
    gpu::upload_model(ctx, seq_model, num_timesteps);
    gpu::upload_dye_tracks(ctx, num_timesteps, num_channels, *dye_tracks);
}

NNClassifier::~NNClassifier() {}

std::vector<ScoredClassification> NNClassifier::classify(const Radiometry& radiometry, unsigned int h) {
    std::vector<ScoredClassification> out;
    if (h == 0) return out;
    std::vector<int32_t> ncand(1), ids(h);
    std::vector<double> scores(h), total(1);
    ctx.check(wp_nn_classify(ctx.get(), radiometry.intensities, 1, k, sig, (int)h, ncand.data(), ids.data(),
                             scores.data(), total.data()),
              "wp_nn_classify");
    for (int i = 0; i < ncand[0]; i++) out.push_back(ScoredClassification(ids[i], scores[i], total[0]));
    return out;
}

ScoredClassification NNClassifier::classify(const Radiometry& radiometry) {
    std::vector<ScoredClassification> top = classify(radiometry, 1u);
    if (top.empty()) return gpu::patched(-1, -1.0, 0.0);
    return gpu::patched(top[0].id, top[0].score, top[0].total);
}

std::vector<ScoredClassification> NNClassifier::classify(const std::vector<Radiometry>& radiometries) {
    const int R = (int)radiometries.size();
    std::vector<ScoredClassification> out;
    if (R == 0) return out;
    const std::vector<double> rads = gpu::flatten(radiometries);
    std::vector<int32_t> ncand(R), ids(R);
    std::vector<double> scores(R), total(R);
    ctx.check(wp_nn_classify(ctx.get(), rads.data(), R, k, sig, 1, ncand.data(), ids.data(), scores.data(),
                             total.data()),
              "wp_nn_classify");
    out.reserve(R);
    for (int r = 0; r < R; r++)
        out.push_back(ncand[r] > 0 ? gpu::patched(ids[r], scores[r], total[r]) : gpu::patched(-1, -1.0, total[r]));
    return out;
}

// ---------------------------------------------------------------- HybridClassifier

HybridClassifier::HybridClassifier(unsigned int num_timesteps,
                                   unsigned int num_channels,
                                   const SequencingModel& seq_model,
                                   const SequencingSettings& seq_settings,
                                   int k,
                                   double sig,
                                   std::vector<SourcedData<DyeTrack, SourceCountHitsList<int>>>* dye_tracks,
                                   int h,
                                   const std::vector<SourcedData<DyeSeq, SourceCount<int>>>& dye_seqs)
        : h(h),
          num_timesteps(num_timesteps),
          num_channels(num_channels),
          k(k),
          sig(sig),
          dist_cutoff(seq_settings.dist_cutoff) {
    gpu::upload_model(ctx, seq_model, num_timesteps);
    gpu::upload_dye_seqs(ctx, dye_seqs);
    gpu::upload_dye_tracks(ctx, num_timesteps, num_channels, *dye_tracks);
}

std::vector<ScoredClassification> HybridClassifier::run(const double* rads, int num_reads) {
    std::vector<int32_t> id(num_reads);
    std::vector<double> score(num_reads), total(num_reads);
    if (num_reads > 0)
        ctx.check(wp_hybrid_classify(ctx.get(), rads, num_reads, k, sig, h, dist_cutoff, id.data(), score.data(),
                                     total.data()),
                  "wp_hybrid_classify");
    std::vector<ScoredClassification> out;
    out.reserve(num_reads);
    for (int r = 0; r < num_reads; r++) out.push_back(ScoredClassification(id[r], score[r], total[r]));
    return out;
}

ScoredClassification HybridClassifier::classify(const Radiometry& radiometry) {
    return run(radiometry.intensities, 1)[0];
}

std::vector<ScoredClassification> HybridClassifier::classify(const std::vector<Radiometry>& radiometries) {
    const std::vector<double> rads = gpu::flatten(radiometries);
    return run(rads.data(), (int)radiometries.size());
}

// ---------------------------------------------------------------- HMMFitter

HMMFitter::HMMFitter(unsigned int num_timesteps,
                     unsigned int num_channels,
                     double stopping_threshold,
                     double max_runtime,
                     const SequencingModel& seq_model,
                     const SequencingSettings& seq_settings,
                     const FitSettings& fit_settings,
                     const DyeSeq& dye_seq)
        : dye_seq(dye_seq),
          seq_model(seq_model),
          seq_settings(seq_settings),
          fit_settings(fit_settings),
          stopping_threshold(stopping_threshold),
          max_runtime(max_runtime),
          num_timesteps(num_timesteps),
          num_channels(num_channels) {}

double HMMFitter::fit_flat(const double* rads, int num_reads, SequencingModel* x, double* step_size) const {
    if (seq_settings.dist_cutoff < DBL_MAX)
        throw std::invalid_argument(
                "whatprot_gpu: HMMFitter fits unpruned; set SequencingSettings::dist_cutoff to the largest double");
    gpu::ModelArrays start(seq_model);
    wp_fit_settings fs = {};
    fs.hold_p_edman_failure = fit_settings.hold_p_edman_failure;
    fs.hold_p_detach = fit_settings.hold_p_detach;
    fs.hold_p_initial_detach = fit_settings.hold_p_initial_detach;
    fs.hold_p_initial_detach_decay = fit_settings.hold_p_initial_detach_decay;
    fs.hold_p_initial_block = fit_settings.hold_p_initial_block;
    fs.hold_p_cyclic_block = fit_settings.hold_p_cyclic_block;
    for (size_t c = 0; c < fit_settings.channel_fit_settings.size() && c < WP_MAX_CHANNELS; c++) {
        fs.hold_p_bleach[c] = fit_settings.channel_fit_settings[c]->hold_p_bleach;
        fs.hold_p_dud[c] = fit_settings.channel_fit_settings[c]->hold_p_dud;
    }
    const std::vector<int16_t> seq = gpu::dye_seq_array(dye_seq);
    wp_fit_params out;
    double step = 0.0, log_l = 0.0;
    ctx.check(wp_hmm_fit(ctx.get(), &start.m, (int)num_timesteps, seq.empty() ? nullptr : seq.data(),
                         (int)seq.size(), rads, num_reads, &fs, stopping_threshold, max_runtime, &out, &step, &log_l,
                         nullptr),
              "wp_hmm_fit");
    *x = seq_model;
    x->p_edman_failure = out.p_edman_failure;
    x->p_detach.base = out.p_detach;
    x->p_detach.initial = out.p_initial_detach;
    x->p_detach.initial_decay = out.p_initial_detach_decay;
    x->p_initial_block = out.p_initial_block;
    x->p_cyclic_block = out.p_cyclic_block;
    for (size_t c = 0; c < x->channel_models.size() && c < WP_MAX_CHANNELS; c++) {
        x->channel_models[c]->p_bleach = out.p_bleach[c];
        x->channel_models[c]->p_dud = out.p_dud[c];
    }
    *step_size = step;
    return log_l;
}

double HMMFitter::log_likelihood_flat(const double* rads, int num_reads, const SequencingModel& model) const {
    gpu::upload_model(ctx, model, num_timesteps);
    const std::vector<int16_t> seq = gpu::dye_seq_array(dye_seq);
    const int16_t none = -1;
    const int32_t off[2] = {0, (int32_t)seq.size()}, id = 0, count = 1;
    ctx.check(wp_peptides_upload(ctx.get(), seq.empty() ? &none : seq.data(), off, &id, &count, 1),
              "wp_peptides_upload");
    std::vector<double> logp(num_reads);
    if (num_reads > 0)
        ctx.check(wp_hmm_loglik_all(ctx.get(), rads, num_reads, seq_settings.dist_cutoff, logp.data()),
                  "wp_hmm_loglik_all");
    double sum = 0.0;
    for (double v : logp) sum += v;
    return sum;
}

}  // namespace whatprot

// whatprot_gpu.h -- whatprot's classifier and fitter classes, run on the GPU.
//
// Drop-in replacements for
//   HMMClassifier     classifiers/hmm-classifier.h:32-43
//   NNClassifier      classifiers/nn-classifier.h:58-82
//   HybridClassifier  classifiers/hybrid-classifier.h:31-44
//   HMMFitter         fitters/hmm-fitter.h:35-142
// (paths relative to whatprot's cc_code/src/): the same namespace, class
// names, constructors and public methods, implemented over the C ABI of
// include/whatprot_gb300.h instead of the per-pair CPU HMM.  A program that
// includes these four headers includes this one instead and links
// whatprot_gpu.cc and libwhatprot_gb300.so; nothing else changes.
//
// Differences a caller can see:
//   * batches: classify(vector) is one GPU batch (no OpenMP loop);
//   * errors: a failed GPU call throws std::runtime_error carrying the
//     library's message (the CPU classes have no failure path);
//   * the dye-tracks: NNClassifier and HybridClassifier copy them to the
//     device and leave the caller's vector as it was (whatprot's
//     NNClassifier moves them into its kd-tree);
//   * HMMFitter::fit runs unpruned, as `whatprot fit` does
//     (main/run-fit.cc:59); a finite SequencingSettings::dist_cutoff is
//     rejected (std::invalid_argument);
//   * internals (the precomputations, the kd-tree, the nested classifiers
//     of HybridClassifier) are not members.
// The device is WHATPROT_GPU_DEVICE (an integer, default 0).  Each object
// owns one device context; an object is used from one thread at a time.
#ifndef WHATPROT_GPU_H
#define WHATPROT_GPU_H

#include <string>
#include <vector>

#ifdef WHATPROT_GPU_WITH_REFERENCE
#include "common/dye-seq.h"
#include "common/dye-track.h"
#include "common/radiometry.h"
#include "common/scored-classification.h"
#include "common/sourced-data.h"
#include "parameterization/model/sequencing-model.h"
#include "parameterization/settings/fit-settings.h"
#include "parameterization/settings/sequencing-settings.h"
#else
#include "whatprot_types.h"
#endif

struct wp_ctx;

namespace whatprot {

namespace gpu {

// One device context (wp_ctx_create / wp_ctx_destroy).
class Context {
public:
    Context();
    ~Context();
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    wp_ctx* get() const { return ctx_; }
    // Throws std::runtime_error with the library's message unless st == 0.
    void check(int st, const char* what) const;

private:
    wp_ctx* ctx_;
};

// Reads [R][T][C] as one contiguous host array.
std::vector<double> flatten(const std::vector<Radiometry>& radiometries);
std::vector<double> flatten(const std::vector<Radiometry*>& radiometries);
std::vector<double> flatten(const std::vector<const Radiometry*>& radiometries);

void upload_model(const Context& ctx, const SequencingModel& seq_model, unsigned int num_timesteps);
void upload_dye_seqs(const Context& ctx, const std::vector<SourcedData<DyeSeq, SourceCount<int>>>& dye_seqs);
void upload_dye_tracks(const Context& ctx, unsigned int num_timesteps, unsigned int num_channels,
                       const std::vector<SourcedData<DyeTrack, SourceCountHitsList<int>>>& dye_tracks);

}  // namespace gpu

class HMMClassifier {
public:
    HMMClassifier(unsigned int num_timesteps,
                  unsigned int num_channels,
                  const SequencingModel& seq_model,
                  const SequencingSettings& seq_settings,
                  const std::vector<SourcedData<DyeSeq, SourceCount<int>>>& dye_seqs);
    ~HMMClassifier();
    ScoredClassification classify(const Radiometry& radiometry);
    // Only the peptides at candidate_indices (indices into dye_seqs); ties go
    // to the first in candidate order.
    ScoredClassification classify(const Radiometry& radiometry, const std::vector<int>& candidate_indices);
    std::vector<ScoredClassification> classify(const std::vector<Radiometry>& radiometries);

    const SequencingModel& seq_model;
    const SequencingSettings& seq_settings;
    const std::vector<SourcedData<DyeSeq, SourceCount<int>>>& dye_seqs;
    unsigned int num_timesteps;
    unsigned int num_channels;
    unsigned int max_num_dyes;

private:
    std::vector<ScoredClassification> run(const double* rads, int num_reads, const int* cand, const int* cand_off);
    gpu::Context ctx;
};

class NNClassifier {
public:
    NNClassifier(unsigned int num_timesteps,
                 unsigned int num_channels,
                 const SequencingModel& seq_model,
                 int k,
                 double sig,
                 std::vector<SourcedData<DyeTrack, SourceCountHitsList<int>>>* dye_tracks);
    ~NNClassifier();
    ScoredClassification classify(const Radiometry& radiometry);
    // The top h peptide ids by kNN score, ascending.
    std::vector<ScoredClassification> classify(const Radiometry& radiometry, unsigned int h);
    std::vector<ScoredClassification> classify(const std::vector<Radiometry>& radiometries);

    int num_train;
    unsigned int num_timesteps;
    unsigned int num_channels;
    int k;
    double two_sig_sq;

private:
    double sig;
    gpu::Context ctx;
};

class HybridClassifier {
public:
    HybridClassifier(unsigned int num_timesteps,
                     unsigned int num_channels,
                     const SequencingModel& seq_model,
                     const SequencingSettings& seq_settings,
                     int k,
                     double sig,
                     std::vector<SourcedData<DyeTrack, SourceCountHitsList<int>>>* dye_tracks,
                     int h,
                     const std::vector<SourcedData<DyeSeq, SourceCount<int>>>& dye_seqs);
    ScoredClassification classify(const Radiometry& radiometry);
    std::vector<ScoredClassification> classify(const std::vector<Radiometry>& radiometries);

    int h;

private:
    std::vector<ScoredClassification> run(const double* rads, int num_reads);
    unsigned int num_timesteps;
    unsigned int num_channels;
    int k;
    double sig;
    double dist_cutoff;
    gpu::Context ctx;
};

class HMMFitter {
public:
    HMMFitter(unsigned int num_timesteps,
              unsigned int num_channels,
              double stopping_threshold,
              double max_runtime,
              const SequencingModel& seq_model,
              const SequencingSettings& seq_settings,
              const FitSettings& fit_settings,
              const DyeSeq& dye_seq);

    // Baum-Welch from seq_model until the step is below stopping_threshold
    // or max_runtime seconds have passed; *x receives the fitted model (a
    // copy of seq_model with the fitted rates), *step_size the last step.
    // Returns the log-likelihood of the reads under *x.  R: Radiometry or a
    // pointer to one.
    template <class R>
    double fit(const std::vector<R>& radiometries, SequencingModel* x, double* step_size) const {
        const std::vector<double> rads = gpu::flatten(radiometries);
        return fit_flat(rads.data(), (int)radiometries.size(), x, step_size);
    }

    template <class R>
    double log_likelihood(const std::vector<R>& radiometries, const SequencingModel& model) const {
        const std::vector<double> rads = gpu::flatten(radiometries);
        return log_likelihood_flat(rads.data(), (int)radiometries.size(), model);
    }

    const DyeSeq& dye_seq;
    const SequencingModel& seq_model;
    const SequencingSettings& seq_settings;
    const FitSettings& fit_settings;
    double stopping_threshold;
    double max_runtime;
    unsigned int num_timesteps;
    unsigned int num_channels;

private:
    double fit_flat(const double* rads, int num_reads, SequencingModel* x, double* step_size) const;
    double log_likelihood_flat(const double* rads, int num_reads, const SequencingModel& model) const;
    gpu::Context ctx;
};

}  // namespace whatprot

#endif  // WHATPROT_GPU_H

// whatprot_types.h -- the whatprot data types the GPU classifiers take, for
// builds without the whatprot source tree.
//
// A program that already has whatprot's own headers compiles
// whatprot_gpu.cc with -DWHATPROT_GPU_WITH_REFERENCE and its include path
// (cc_code/src), and this file is not used.  Otherwise this file declares
// the same classes with the same public members, so that code written
// against whatprot's classifier interfaces compiles unchanged:
//
//   Radiometry            common/radiometry.h          intensities[t * C + c]
//   DyeSeq                common/dye-seq.h             seq[i]: -1 or a channel
//   DyeTrack              common/dye-track.h           counts[t * C + c]
//   SourcedData, SourceCount, SourceCountHits, SourceCountHitsList
//                         common/sourced-data.h        owning containers
//   ScoredClassification  common/scored-classification.h
//   ChannelModel, DecayingRateModel, SequencingModel
//                         parameterization/model/*.h   rates and channel models
//   SequencingSettings, ChannelFitSettings, FitSettings
//                         parameterization/settings/*.h
//
// Only what the classifiers and the fitter read is here: no file readers,
// no pdf or distance helpers beyond SequencingModel::distance.
#ifndef WHATPROT_GPU_TYPES_H
#define WHATPROT_GPU_TYPES_H

#include <algorithm>
#include <cmath>
#include <string>
#include <utility>
#include <vector>

namespace whatprot {

class Radiometry {
public:
    Radiometry(unsigned int num_timesteps, unsigned int num_channels)
            : intensities(new double[num_timesteps * num_channels]()),
              num_timesteps(num_timesteps),
              num_channels(num_channels) {}
    Radiometry(const Radiometry& o) : Radiometry(o.num_timesteps, o.num_channels) {
        std::copy(o.intensities, o.intensities + num_timesteps * num_channels, intensities);
    }
    Radiometry& operator=(const Radiometry& o) {
        if (this != &o) {
            Radiometry tmp(o);
            std::swap(intensities, tmp.intensities);
            num_timesteps = o.num_timesteps;
            num_channels = o.num_channels;
        }
        return *this;
    }
    ~Radiometry() { delete[] intensities; }
    double& operator()(int t, int c) { return intensities[t * num_channels + c]; }
    double operator()(int t, int c) const { return intensities[t * num_channels + c]; }

    double* intensities;
    unsigned int num_timesteps;
    unsigned int num_channels;
};

class DyeSeq {
public:
    // s: '.' for an unlabeled position, a digit for the channel of a dye;
    // trailing '.' are dropped.
    DyeSeq(unsigned int num_channels, const std::string& s) : num_channels(num_channels) {
        length = (unsigned int)s.size();
        while (length > 0 && s[length - 1] == '.') length--;
        seq = new short[length];
        for (unsigned int i = 0; i < length; i++) seq[i] = s[i] == '.' ? (short)-1 : (short)(s[i] - '0');
    }
    DyeSeq(const DyeSeq& o) : seq(new short[o.length]), length(o.length), num_channels(o.num_channels) {
        std::copy(o.seq, o.seq + length, seq);
    }
    ~DyeSeq() { delete[] seq; }
    short operator[](unsigned int i) const { return i < length ? seq[i] : (short)-1; }
    short& operator[](unsigned int i) { return seq[i]; }

    short* seq;
    unsigned int length;
    unsigned int num_channels;
};

class DyeTrack {
public:
    DyeTrack(unsigned int num_timesteps, unsigned int num_channels)
            : counts((size_t)num_timesteps * num_channels, 0),
              num_timesteps(num_timesteps),
              num_channels(num_channels) {}
    short& operator()(int t, int c) { return counts[t * num_channels + c]; }
    short operator()(int t, int c) const { return counts[t * num_channels + c]; }

    std::vector<short> counts;
    unsigned int num_timesteps;
    unsigned int num_channels;
};

template <typename S>
class SourceCount {
public:
    SourceCount(S source, int count) : source(source), count(count) {}
    S source;
    int count;
};

template <typename S>
class SourceCountHits {
public:
    SourceCountHits(S source, int count, int hits) : source(source), count(count), hits(hits) {}
    S source;
    int count;
    int hits;
};

// Owns its sources (each allocated with new, the array with new[]).
template <typename S>
class SourceCountHitsList {
public:
    SourceCountHitsList(int num_sources, SourceCountHits<S>** sources) : sources(sources), num_sources(num_sources) {}
    SourceCountHitsList(SourceCountHitsList&& o) : sources(o.sources), num_sources(o.num_sources) {
        o.sources = nullptr;
        o.num_sources = 0;
    }
    SourceCountHitsList(const SourceCountHitsList&) = delete;
    ~SourceCountHitsList() {
        if (!sources) return;
        for (int i = 0; i < num_sources; i++) delete sources[i];
        delete[] sources;
    }
    SourceCountHits<S>** sources;
    int num_sources;
};

template <typename V, typename S>
class SourcedData {
public:
    SourcedData(V value, S source) : value(std::move(value)), source(std::move(source)) {}
    SourcedData(SourcedData&& o) : value(std::move(o.value)), source(std::move(o.source)) {}
    V value;
    S source;
};

class ScoredClassification {
public:
    ScoredClassification() : score(-2147483648.0), total(0.0), id(-1) {}
    ScoredClassification(int id, double score, double total) : score(score), total(total), id(id) {}
    double adjusted_score() const { return score / total; }
    double score;
    double total;
    int id;
};

class ChannelModel {
public:
    ChannelModel(unsigned int channel, unsigned int num_channels)
            : channel(channel),
              num_channels(num_channels),
              p_bleach(0.0),
              p_dud(0.0),
              bg_sig(0.0),
              mu(1.0),
              sig(0.0),
              interactions(num_channels, 1.0),
              flat_interactions(num_channels, 1.0) {}
    virtual ~ChannelModel() {}
    unsigned int channel;
    unsigned int num_channels;
    double p_bleach;
    double p_dud;
    double bg_sig;
    double mu;
    double sig;
    std::vector<double> interactions;
    std::vector<double> flat_interactions;
};

// Rate base + initial * exp(-initial_decay * t) at timestep t.
class DecayingRateModel {
public:
    DecayingRateModel() : base(0.0), initial(0.0), initial_decay(0.0) {}
    double operator[](unsigned int t) const { return base + initial * std::exp(-initial_decay * (double)t); }
    double base;
    double initial;
    double initial_decay;
};

// Owns its channel models (deep copies on copy and assignment).
class SequencingModel {
public:
    SequencingModel() : p_edman_failure(0.0), p_initial_block(0.0), p_cyclic_block(0.0) {}
    explicit SequencingModel(unsigned int num_channels) : SequencingModel() {
        for (unsigned int c = 0; c < num_channels; c++) channel_models.push_back(new ChannelModel(c, num_channels));
    }
    SequencingModel(const SequencingModel& o) { *this = o; }
    SequencingModel& operator=(const SequencingModel& o) {
        if (this == &o) return *this;
        for (ChannelModel* cm : channel_models) delete cm;
        channel_models.clear();
        p_edman_failure = o.p_edman_failure;
        p_detach = o.p_detach;
        p_initial_block = o.p_initial_block;
        p_cyclic_block = o.p_cyclic_block;
        for (const ChannelModel* cm : o.channel_models) channel_models.push_back(new ChannelModel(*cm));
        return *this;
    }
    ~SequencingModel() {
        for (ChannelModel* cm : channel_models) delete cm;
    }
    // The largest absolute change of a fitted rate.
    double distance(const SequencingModel& o) const {
        double d = std::max({std::fabs(p_edman_failure - o.p_edman_failure), std::fabs(p_detach.base - o.p_detach.base),
                             std::fabs(p_detach.initial - o.p_detach.initial),
                             std::fabs(p_detach.initial_decay - o.p_detach.initial_decay),
                             std::fabs(p_initial_block - o.p_initial_block),
                             std::fabs(p_cyclic_block - o.p_cyclic_block)});
        for (size_t c = 0; c < channel_models.size() && c < o.channel_models.size(); c++)
            d = std::max({d, std::fabs(channel_models[c]->p_bleach - o.channel_models[c]->p_bleach),
                          std::fabs(channel_models[c]->p_dud - o.channel_models[c]->p_dud)});
        return d;
    }
    double p_edman_failure;
    DecayingRateModel p_detach;
    double p_initial_block;
    double p_cyclic_block;
    std::vector<ChannelModel*> channel_models;
};

class SequencingSettings {
public:
    double dist_cutoff;  // emission pruning, in standard deviations
};

class ChannelFitSettings {
public:
    ChannelFitSettings() : hold_p_bleach(false), hold_p_dud(false) {}
    bool hold_p_bleach;
    bool hold_p_dud;
};

// Owns its channel settings.
class FitSettings {
public:
    FitSettings()
            : hold_p_edman_failure(false),
              hold_p_detach(false),
              hold_p_initial_detach(false),
              hold_p_initial_detach_decay(false),
              hold_p_initial_block(false),
              hold_p_cyclic_block(false) {}
    explicit FitSettings(unsigned int num_channels) : FitSettings() {
        for (unsigned int c = 0; c < num_channels; c++) channel_fit_settings.push_back(new ChannelFitSettings());
    }
    FitSettings(const FitSettings&) = delete;
    ~FitSettings() {
        for (ChannelFitSettings* s : channel_fit_settings) delete s;
    }
    bool hold_p_edman_failure;
    bool hold_p_detach;
    bool hold_p_initial_detach;
    bool hold_p_initial_detach_decay;
    bool hold_p_initial_block;
    bool hold_p_cyclic_block;
    std::vector<ChannelFitSettings*> channel_fit_settings;
};

}  // namespace whatprot

#endif  // WHATPROT_GPU_TYPES_H

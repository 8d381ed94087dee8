// dropin_driver.cc -- drives the GPU drop-in classes (whatprot_gpu.h) the
// way whatprot's run-classify-*.cc and run-fit.cc drive the CPU ones, on
// inputs given as a plain token file, and prints the results.  Test
// program for tests/test_gpu_cpp_dropin.py; it compiles against the
// library's own data types or, with -DWHATPROT_GPU_WITH_REFERENCE, against
// whatprot's headers.
//
//   dropin_driver <hmm|nn|hybrid|fit> <input file>
//
// Input tokens (whitespace separated):
//   C T cutoff                       (cutoff "max": the largest double)
//   p_edman_failure p_detach p_initial_detach p_initial_detach_decay
//   p_initial_block p_cyclic_block
//   C x (p_bleach p_dud bg_sig mu sig)
//   P, then P x (id count dye-string)          ("-" for an empty string)
//   N, then N x (T*C counts, nsrc, nsrc x (id count hits))
//   k sig h
//   R, then R x (T*C intensities)
//   fit only: threshold dye-string
// Output: one line per read "id score total" (%.17g), or for fit the fitted
// p_edman_failure p_detach p_initial_detach p_initial_detach_decay
// p_initial_block p_cyclic_block, C x p_bleach, C x p_dud, then log_l and
// step size.  Exit status 3: a library call failed (message on stderr).
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <string>
#include <vector>

#include "whatprot_gpu.h"

using namespace whatprot;

namespace {

double num(std::ifstream& f) {
    std::string s;
    f >> s;
    if (s == "max") return DBL_MAX;
    return std::strtod(s.c_str(), nullptr);
}

std::string seq_str(std::ifstream& f) {
    std::string s;
    f >> s;
    return s == "-" ? std::string() : s;
}

int run(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <hmm|nn|hybrid|fit> <input>\n", argv[0]);
        return 2;
    }
    const std::string mode = argv[1];
    std::ifstream f(argv[2]);
    const unsigned int C = (unsigned int)num(f), T = (unsigned int)num(f);
    SequencingSettings settings;
    settings.dist_cutoff = num(f);
    SequencingModel sm(C);
    sm.p_edman_failure = num(f);
    sm.p_detach.base = num(f);
    sm.p_detach.initial = num(f);
    sm.p_detach.initial_decay = num(f);
    sm.p_initial_block = num(f);
    sm.p_cyclic_block = num(f);
    for (unsigned int c = 0; c < C; c++) {
        ChannelModel& cm = *sm.channel_models[c];
        cm.p_bleach = num(f);
        cm.p_dud = num(f);
        cm.bg_sig = num(f);
        cm.mu = num(f);
        cm.sig = num(f);
    }
    std::vector<SourcedData<DyeSeq, SourceCount<int>>> dye_seqs;
    const int P = (int)num(f);
    for (int i = 0; i < P; i++) {
        const int id = (int)num(f), count = (int)num(f);
        dye_seqs.push_back(SourcedData<DyeSeq, SourceCount<int>>(DyeSeq(C, seq_str(f)), SourceCount<int>(id, count)));
    }
    std::vector<SourcedData<DyeTrack, SourceCountHitsList<int>>> dye_tracks;
    const int N = (int)num(f);
    for (int e = 0; e < N; e++) {
        DyeTrack track(T, C);
        for (unsigned int i = 0; i < T * C; i++) track.counts[i] = (short)num(f);
        const int ns = (int)num(f);
        SourceCountHits<int>** src = new SourceCountHits<int>*[ns];
        for (int j = 0; j < ns; j++) {
            const int id = (int)num(f), count = (int)num(f), hits = (int)num(f);
            src[j] = new SourceCountHits<int>(id, count, hits);
        }
        dye_tracks.push_back(SourcedData<DyeTrack, SourceCountHitsList<int>>(std::move(track),
                                                                           SourceCountHitsList<int>(ns, src)));
    }
    const int k = (int)num(f);
    const double sig = num(f);
    const int h = (int)num(f);
    std::vector<Radiometry> rads;
    const int R = (int)num(f);
    rads.reserve(R);
    for (int r = 0; r < R; r++) {
        Radiometry rad(T, C);
        for (unsigned int i = 0; i < T * C; i++) rad.intensities[i] = num(f);
        rads.push_back(rad);
    }
    std::vector<ScoredClassification> out;
    if (mode == "hmm") {
        HMMClassifier classifier(T, C, sm, settings, dye_seqs);
        out = classifier.classify(rads);
        // the single-read and candidate overloads agree with the batch
        if (R > 0) {
            ScoredClassification one = classifier.classify(rads[0]);
            std::vector<int> all;
            for (int i = 0; i < P; i++) all.push_back(i);
            ScoredClassification cand = classifier.classify(rads[0], all);
            if (one.id != out[0].id || cand.id != out[0].id) {
                std::fprintf(stderr, "overloads disagree\n");
                return 1;
            }
        }
    } else if (mode == "nn") {
        NNClassifier classifier(T, C, sm, k, sig, &dye_tracks);
        out = classifier.classify(rads);
    } else if (mode == "hybrid") {
        HybridClassifier classifier(T, C, sm, settings, k, sig, &dye_tracks, h, dye_seqs);
        out = classifier.classify(rads);
    } else if (mode == "fit") {
        const double threshold = num(f);
        DyeSeq dye_seq(C, seq_str(f));
        FitSettings fit_settings(C);
        HMMFitter fitter(T, C, threshold, 1e9, sm, settings, fit_settings, dye_seq);
        SequencingModel fitted;
        double step = 0.0;
        const double log_l = fitter.fit(rads, &fitted, &step);
        std::printf("%.17g %.17g %.17g %.17g %.17g %.17g", fitted.p_edman_failure, fitted.p_detach.base,
                    fitted.p_detach.initial, fitted.p_detach.initial_decay, fitted.p_initial_block,
                    fitted.p_cyclic_block);
        for (unsigned int c = 0; c < C; c++) std::printf(" %.17g", fitted.channel_models[c]->p_bleach);
        for (unsigned int c = 0; c < C; c++) std::printf(" %.17g", fitted.channel_models[c]->p_dud);
        std::printf(" %.17g %.17g\n", log_l, step);
        std::printf("log_likelihood %.17g\n", fitter.log_likelihood(rads, fitted));
        return 0;
    } else {
        std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
        return 2;
    }
    for (const ScoredClassification& s : out) std::printf("%d %.17g %.17g\n", s.id, s.score, s.total);
    return 0;
}

}  // namespace

// A failed GPU call surfaces as an exception: exit status 3 with its message.
int main(int argc, char** argv) {
    try {
        return run(argc, argv);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 3;
    }
}

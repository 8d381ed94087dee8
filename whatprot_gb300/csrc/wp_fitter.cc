// wp_fitter.cc -- the host side of the Baum-Welch fit: HMMFitter::fit
// (fitters/hmm-fitter.h:49-117) as a client of the C ABI.  Each iteration
// uploads the current model, runs one GPU E-step over the staged reads
// (wp_fit_estep), applies the dud hidden-count correction and the M-step on
// the host, and stops on the largest parameter change or on wall time.
//
// The detach M-step fits base + initial * exp(-decay * t) by weighted least
// squares with every parameter in [0, 1] (util/levmar-helper.cc:44-85).  The
// reference calls levmar's box-constrained dlevmar_bc_der (levmar 2.6,
// vendored by the reference); this file has its own projected
// Levenberg-Marquardt (Levenberg 1944, Marquardt 1963; damping update of
// Nielsen 1999) with the same bounds, the same 10-iteration cap and holds as
// fixed parameters, so fitted detach rates agree with the reference to the
// accuracy of the fit, not bit for bit.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <random>
#include <vector>

#include "whatprot_gb300.h"

wp_status wp_internal_fail(wp_ctx* ctx, wp_status code, const char* msg);

namespace {

// Model of offset_exponential (util/levmar-helper.cc:23-42), weighted.
void oe_residual(const double* p, const double* y, const double* sw, int n, double* r) {
    for (int i = 0; i < n; i++) r[i] = sw[i] * (y[i] - (p[0] + p[1] * exp(-p[2] * i)));
}

void oe_normal(const double* p, const double* sw, const double* r, int n, double A[3][3], double g[3]) {
    for (int a = 0; a < 3; a++) {
        g[a] = 0.0;
        for (int b = 0; b < 3; b++) A[a][b] = 0.0;
    }
    for (int i = 0; i < n; i++) {
        const double e = exp(-p[2] * i);
        const double J[3] = {sw[i], sw[i] * e, -sw[i] * p[1] * i * e};
        for (int a = 0; a < 3; a++) {
            g[a] += J[a] * r[i];
            for (int b = 0; b < 3; b++) A[a][b] += J[a] * J[b];
        }
    }
}

double sumsq(const double* r, int n) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += r[i] * r[i];
    return s;
}

// Solve M h = g on the free coordinates by Cholesky (M symmetric positive
// definite there); fixed coordinates get h = 0.  False if M is not SPD.
bool solve_free(const double M[3][3], const double g[3], const bool* fixed, double h[3]) {
    int idx[3], m = 0;
    for (int k = 0; k < 3; k++) {
        h[k] = 0.0;
        if (!fixed[k]) idx[m++] = k;
    }
    double L[3][3] = {{0}};
    for (int i = 0; i < m; i++) {
        for (int j = 0; j <= i; j++) {
            double s = M[idx[i]][idx[j]];
            for (int k = 0; k < j; k++) s -= L[i][k] * L[j][k];
            if (i == j) {
                if (!(s > 0.0)) return false;
                L[i][i] = sqrt(s);
            } else {
                L[i][j] = s / L[j][j];
            }
        }
    }
    double z[3];
    for (int i = 0; i < m; i++) {
        double s = g[idx[i]];
        for (int k = 0; k < i; k++) s -= L[i][k] * z[k];
        z[i] = s / L[i][i];
    }
    for (int i = m - 1; i >= 0; i--) {
        double s = z[i];
        for (int k = i + 1; k < m; k++) s -= L[k][i] * h[idx[k]];
        h[idx[i]] = s / L[i][i];
    }
    return true;
}

struct HostModel {
    int C = 0;
    double p_edman_failure = 0, p_detach = 0, p_initial_detach = 0, p_initial_detach_decay = 0;
    double p_initial_block = 0, p_cyclic_block = 0;
    double p_bleach[WP_MAX_CHANNELS] = {0}, p_dud[WP_MAX_CHANNELS] = {0};
    double bg_sig[WP_MAX_CHANNELS] = {0}, mu[WP_MAX_CHANNELS] = {0}, sig[WP_MAX_CHANNELS] = {0};
    std::vector<double> inter, flat;

    wp_seq_model view() const {
        wp_seq_model m;
        m.num_channels = C;
        m.p_edman_failure = p_edman_failure;
        m.p_detach = p_detach;
        m.p_initial_detach = p_initial_detach;
        m.p_initial_detach_decay = p_initial_detach_decay;
        m.p_initial_block = p_initial_block;
        m.p_cyclic_block = p_cyclic_block;
        m.p_bleach = p_bleach;
        m.p_dud = p_dud;
        m.bg_sig = bg_sig;
        m.mu = mu;
        m.sig = sig;
        m.interactions = inter.empty() ? nullptr : inter.data();
        m.flat_interactions = flat.empty() ? nullptr : flat.data();
        return m;
    }
};

// SequencingModel::distance (parameterization/model/sequencing-model.cc:153-166).
double distance(const HostModel& a, const HostModel& b) {
    double d = 0.0;
    d = std::max(d, fabs(a.p_edman_failure - b.p_edman_failure));
    d = std::max(d, fabs(a.p_detach - b.p_detach));
    d = std::max(d, fabs(a.p_initial_detach - b.p_initial_detach));
    d = std::max(d, fabs(a.p_initial_detach_decay - b.p_initial_detach_decay));
    d = std::max(d, fabs(a.p_initial_block - b.p_initial_block));
    d = std::max(d, fabs(a.p_cyclic_block - b.p_cyclic_block));
    for (int c = 0; c < a.C; c++) {
        d = std::max(d, fabs(a.p_bleach[c] - b.p_bleach[c]));
        d = std::max(d, fabs(a.p_dud[c] - b.p_dud[c]));
    }
    return d;
}

// Expected log-likelihood (up to a constant) of one channel's intensities
// given the emission statistics w, x, xx over dye counts n < nmax, at
// th = (log mu, log sig, log bg_sig), and its gradient in th (nullable).
double emission_q(const double* w, const double* x, const double* xx, int nmax, const double th[3], double g[3]) {
    const double mu = exp(th[0]), sg = exp(th[1]), bg = exp(th[2]);
    double q = 0.0, gmu = 0.0, gsg = 0.0, gbg = 0.0;
    for (int n = 0; n < nmax; n++) {
        if (!(w[n] > 0.0)) continue;
        const double m = mu * n, v = bg * bg + mu * n * sg * sg;
        const double r = xx[n] - 2.0 * m * x[n] + m * m * w[n];
        q += -0.5 * w[n] * log(v) - r / (2.0 * v);
        const double dm = (x[n] - m * w[n]) / v;            // dq / dm_n
        const double dv = -0.5 * w[n] / v + r / (2.0 * v * v);  // dq / dv_n
        gmu += n * dm + n * sg * sg * dv;
        gsg += 2.0 * mu * n * sg * dv;
        gbg += 2.0 * bg * dv;
    }
    if (g) {
        g[0] = mu * gmu;
        g[1] = sg * gsg;
        g[2] = bg * gbg;
    }
    return q;
}

// Maximises emission_q over th from its current value: damped Newton
// (Levenberg 1944 damping on the negated Hessian, which comes from central
// differences of the analytic gradient), fixed coordinates left alone.
void emission_fit_channel(const double* w, const double* x, const double* xx, int nmax, double th[3],
                          const bool fixed[3]) {
    if (fixed[0] && fixed[1] && fixed[2]) return;
    double lambda = 1e-3;
    double g[3];
    double q = emission_q(w, x, xx, nmax, th, g);
    if (!isfinite(q)) return;
    for (int it = 0; it < 200; it++) {
        double H[3][3];
        const double h = 1e-5;
        for (int k = 0; k < 3; k++) {
            double tp[3] = {th[0], th[1], th[2]}, tm[3] = {th[0], th[1], th[2]};
            tp[k] += h;
            tm[k] -= h;
            double gp[3], gm[3];
            emission_q(w, x, xx, nmax, tp, gp);
            emission_q(w, x, xx, nmax, tm, gm);
            for (int a = 0; a < 3; a++) H[a][k] = (gp[a] - gm[a]) / (2.0 * h);
        }
        bool moved = false;
        while (lambda < 1e12) {
            double M[3][3];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) M[a][b] = -0.5 * (H[a][b] + H[b][a]);
            for (int a = 0; a < 3; a++) M[a][a] += lambda * std::max(fabs(M[a][a]), 1e-12);
            double d[3];
            if (solve_free(M, g, fixed, d)) {
                const double tn[3] = {th[0] + d[0], th[1] + d[1], th[2] + d[2]};
                double gn[3];
                const double qn = emission_q(w, x, xx, nmax, tn, gn);
                if (isfinite(qn) && qn >= q) {
                    const double dmax = std::max(fabs(d[0]), std::max(fabs(d[1]), fabs(d[2])));
                    for (int k = 0; k < 3; k++) th[k] = tn[k], g[k] = gn[k];
                    q = qn;
                    lambda = std::max(lambda * 0.1, 1e-12);
                    moved = dmax > 1e-13;
                    break;
                }
            }
            lambda *= 10.0;
        }
        if (!moved) break;
    }
}

wp_fit_params to_params(const HostModel& m) {
    wp_fit_params p;
    memset(&p, 0, sizeof(p));
    p.p_edman_failure = m.p_edman_failure;
    p.p_detach = m.p_detach;
    p.p_initial_detach = m.p_initial_detach;
    p.p_initial_detach_decay = m.p_initial_detach_decay;
    p.p_initial_block = m.p_initial_block;
    p.p_cyclic_block = m.p_cyclic_block;
    for (int c = 0; c < m.C; c++) {
        p.p_bleach[c] = m.p_bleach[c];
        p.p_dud[c] = m.p_dud[c];
        p.mu[c] = m.mu[c];
        p.sig[c] = m.sig[c];
        p.bg_sig[c] = m.bg_sig[c];
    }
    return p;
}

void from_params(const wp_fit_params& p, HostModel* m) {
    m->p_edman_failure = p.p_edman_failure;
    m->p_detach = p.p_detach;
    m->p_initial_detach = p.p_initial_detach;
    m->p_initial_detach_decay = p.p_initial_detach_decay;
    m->p_initial_block = p.p_initial_block;
    m->p_cyclic_block = p.p_cyclic_block;
    for (int c = 0; c < m->C; c++) {
        m->p_bleach[c] = p.p_bleach[c];
        m->p_dud[c] = p.p_dud[c];
        m->mu[c] = p.mu[c];
        m->sig[c] = p.sig[c];
        m->bg_sig[c] = p.bg_sig[c];
    }
}

}  // namespace

extern "C" {

// One M-step from E-step sums (fitters/hmm-fitter.h:80-116): the dud
// hidden-count correction for num_reads reads, p = num/den, the detach
// curve by bounded least squares, holds, and the step (model distance).
wp_status wp_fit_mstep(const wp_fit_sums* sums_in, int C, int T, const int16_t* dye_seq, int length,
                       long long num_reads, const wp_fit_params* cur, const wp_fit_settings* settings,
                       wp_fit_params* next, double* step_size) {
    if (!sums_in || !cur || !next || C < 1 || C > WP_MAX_CHANNELS || T < 1 || T > WP_MAX_TIMESTEPS || length < 0 ||
        (length > 0 && !dye_seq))
        return WP_ERR_INVALID;
    for (int i = 0; i < length; i++)
        if (dye_seq[i] < -1 || dye_seq[i] >= C) return WP_ERR_INVALID;
    wp_fit_settings fs;
    memset(&fs, 0, sizeof(fs));
    if (settings) fs = *settings;
    wp_fit_sums s = *sums_in;
    // Dud hidden-count correction (fitters/hmm-fitter.h:80-101): the ratio
    // of all-dud peptides, per dye of the dye-seq.
    double ratio = 1.0;
    for (int i = 0; i < length; i++)
        if (dye_seq[i] != -1) ratio *= cur->p_dud[dye_seq[i]];
    const double hidden = (1.0 / (1.0 - ratio) - 1.0) * (double)num_reads;
    for (int i = 0; i < length; i++)
        if (dye_seq[i] != -1) {
            s.p_dud_num[dye_seq[i]] += hidden;
            s.p_dud_den[dye_seq[i]] += hidden;
        }
    // SequencingModelFitter::get (sequencing-model-fitter.cc:68-78), then
    // update_with_holds (hmm-fitter.cc:63-97).
    *next = *cur;
    if (!fs.hold_p_edman_failure) next->p_edman_failure = s.p_edman_failure_num / s.p_edman_failure_den;
    if (!fs.hold_p_initial_block) next->p_initial_block = s.p_initial_block_num / s.p_initial_block_den;
    if (!fs.hold_p_cyclic_block) next->p_cyclic_block = s.p_cyclic_block_num / s.p_cyclic_block_den;
    {
        const int n = T - 1;
        std::vector<double> y(std::max(n, 1)), w(std::max(n, 1));
        for (int k = 0; k < n; k++) {
            y[k] = s.p_detach_x[k] / s.p_detach_n[k];
            w[k] = s.p_detach_n[k];
        }
        double p[3] = {cur->p_detach, cur->p_initial_detach, cur->p_initial_detach_decay};
        const int held[3] = {fs.hold_p_detach, fs.hold_p_initial_detach, fs.hold_p_initial_detach_decay};
        wp_status st = wp_fit_offset_exponential(y.data(), w.data(), n, held, p);
        if (st != WP_OK) return st;
        if (!fs.hold_p_detach) next->p_detach = p[0];
        if (!fs.hold_p_initial_detach) next->p_initial_detach = p[1];
        if (!fs.hold_p_initial_detach_decay) next->p_initial_detach_decay = p[2];
    }
    for (int c = 0; c < C; c++) {
        if (!fs.hold_p_bleach[c]) next->p_bleach[c] = s.p_bleach_num[c] / s.p_bleach_den[c];
        if (!fs.hold_p_dud[c]) next->p_dud[c] = s.p_dud_num[c] / s.p_dud_den[c];
    }
    if (step_size) {
        // SequencingModel::distance (sequencing-model.cc:153-166)
        double d = 0.0;
        d = std::max(d, fabs(cur->p_edman_failure - next->p_edman_failure));
        d = std::max(d, fabs(cur->p_detach - next->p_detach));
        d = std::max(d, fabs(cur->p_initial_detach - next->p_initial_detach));
        d = std::max(d, fabs(cur->p_initial_detach_decay - next->p_initial_detach_decay));
        d = std::max(d, fabs(cur->p_initial_block - next->p_initial_block));
        d = std::max(d, fabs(cur->p_cyclic_block - next->p_cyclic_block));
        for (int c = 0; c < C; c++) {
            d = std::max(d, fabs(cur->p_bleach[c] - next->p_bleach[c]));
            d = std::max(d, fabs(cur->p_dud[c] - next->p_dud[c]));
        }
        *step_size = d;
    }
    return WP_OK;
}

wp_status wp_fit_emission_mstep(const wp_emission_sums* sums, int C, const wp_fit_params* cur, wp_fit_params* next,
                                double* step_size) {
    if (!sums || !cur || !next || C < 1 || C > WP_MAX_CHANNELS) return WP_ERR_INVALID;
    const wp_fit_params in = *cur;
    *next = in;
    double step = 0.0;
    const int nmax = WP_MAX_DYES_PER_CHANNEL + 1;
    for (int c = 0; c < C; c++) {
        double above = 0.0;  // weight at n >= 1: what identifies mu and sig
        for (int n = 1; n < nmax; n++) above += sums->w[c][n];
        const bool fixed[3] = {!(above > 0.0) || !(in.mu[c] > 0.0), !(above > 0.0) || !(in.sig[c] > 0.0),
                               !(in.bg_sig[c] > 0.0)};
        double th[3] = {in.mu[c] > 0.0 ? log(in.mu[c]) : 0.0, in.sig[c] > 0.0 ? log(in.sig[c]) : 0.0,
                        in.bg_sig[c] > 0.0 ? log(in.bg_sig[c]) : 0.0};
        emission_fit_channel(sums->w[c], sums->x[c], sums->xx[c], nmax, th, fixed);
        if (!fixed[0]) next->mu[c] = exp(th[0]);
        if (!fixed[1]) next->sig[c] = exp(th[1]);
        if (!fixed[2]) next->bg_sig[c] = exp(th[2]);
        step = std::max(step, fabs(next->mu[c] - in.mu[c]));
        step = std::max(step, fabs(next->sig[c] - in.sig[c]));
        step = std::max(step, fabs(next->bg_sig[c] - in.bg_sig[c]));
    }
    if (step_size) *step_size = step;
    return WP_OK;
}

wp_status wp_fit_offset_exponential(const double* y, const double* w, int n, const int* held, double* params) {
    if (n < 0 || !params || (n > 0 && (!y || !w))) return WP_ERR_INVALID;
    if (n == 0) return WP_OK;
    double lb[3], ub[3];
    bool fixed[3];
    for (int k = 0; k < 3; k++) {
        fixed[k] = held && held[k];
        lb[k] = fixed[k] ? params[k] : 0.0;
        ub[k] = fixed[k] ? params[k] : 1.0;
    }
    // Weighted problem: residual sqrt(w) * (y - model), as the reference
    // scales both sides by sqrt(w).  Points with a non-finite target or
    // weight carry no information and get weight 0.
    std::vector<double> sw(n), yy(n), r(n), rn(n);
    for (int i = 0; i < n; i++) {
        const bool ok = isfinite(y[i]) && isfinite(w[i]) && w[i] > 0.0;
        sw[i] = ok ? sqrt(w[i]) : 0.0;
        yy[i] = ok ? y[i] : 0.0;
    }
    double p[3];
    for (int k = 0; k < 3; k++) p[k] = std::min(std::max(params[k], lb[k]), ub[k]);
    oe_residual(p, yy.data(), sw.data(), n, r.data());
    double cost = sumsq(r.data(), n);
    double A[3][3], g[3];
    oe_normal(p, sw.data(), r.data(), n, A, g);
    double amax = 0.0;
    for (int k = 0; k < 3; k++)
        if (!fixed[k]) amax = std::max(amax, A[k][k]);
    double mu = 1e-3 * amax;
    double nu = 2.0;
    for (int it = 0; it < 10; it++) {  // itmax of levmar-helper.cc:79
        // Active set: held parameters and those on a bound that the
        // gradient pushes outward stay put this iteration.
        bool act[3];
        double gmax = 0.0;
        for (int k = 0; k < 3; k++) {
            act[k] = fixed[k] || (p[k] <= lb[k] && g[k] <= 0.0) || (p[k] >= ub[k] && g[k] >= 0.0);
            if (!act[k]) gmax = std::max(gmax, fabs(g[k]));
        }
        if (gmax <= 1e-17) break;
        double M[3][3];
        memcpy(M, A, sizeof(M));
        for (int k = 0; k < 3; k++) M[k][k] += mu;
        double h[3];
        if (!solve_free(M, g, act, h)) {
            mu = mu > 0.0 ? mu * nu : 1e-3;
            nu *= 2.0;
            continue;
        }
        double pn[3], d[3], pnorm = 0.0, dnorm = 0.0;
        for (int k = 0; k < 3; k++) {
            pn[k] = std::min(std::max(p[k] + h[k], lb[k]), ub[k]);
            d[k] = pn[k] - p[k];
            pnorm += p[k] * p[k];
            dnorm += d[k] * d[k];
        }
        if (dnorm <= 1e-34 * pnorm) break;
        oe_residual(pn, yy.data(), sw.data(), n, rn.data());
        const double costn = sumsq(rn.data(), n);
        // Reduction predicted by the linearised model along the projected
        // step: |r|^2 - |r - J d|^2 = 2 d.g - d.A.d.
        double pred = 0.0;
        for (int a = 0; a < 3; a++) {
            pred += 2.0 * d[a] * g[a];
            for (int b = 0; b < 3; b++) pred -= d[a] * A[a][b] * d[b];
        }
        const double rho = pred > 0.0 ? (cost - costn) / pred : -1.0;
        if (rho > 0.0 && isfinite(costn)) {
            memcpy(p, pn, sizeof(p));
            r.swap(rn);
            cost = costn;
            oe_normal(p, sw.data(), r.data(), n, A, g);
            const double q = 2.0 * rho - 1.0;
            mu *= std::max(1.0 / 3.0, 1.0 - q * q * q);
            nu = 2.0;
        } else {
            mu *= nu;
            nu *= 2.0;
        }
    }
    for (int k = 0; k < 3; k++) params[k] = p[k];
    return WP_OK;
}

wp_status wp_hmm_fit(wp_ctx* ctx, const wp_seq_model* start, int T, const int16_t* dye_seq, int length,
                     const double* rads, int R, const wp_fit_settings* settings, double stopping_threshold,
                     double max_runtime, wp_fit_params* out, double* step_size, double* log_l, int* iterations) {
    if (!ctx || !start || !out) return WP_ERR_INVALID;
    const int C = start->num_channels;
    if (C < 1 || C > WP_MAX_CHANNELS) return wp_internal_fail(ctx, WP_ERR_UNSUPPORTED, "num_channels out of range 1..4");
    if (!start->p_bleach || !start->p_dud || !start->bg_sig || !start->mu || !start->sig)
        return wp_internal_fail(ctx, WP_ERR_INVALID, "null per-channel array");
    wp_fit_settings fs;
    memset(&fs, 0, sizeof(fs));
    if (settings) fs = *settings;

    HostModel sm;
    sm.C = C;
    sm.p_edman_failure = start->p_edman_failure;
    sm.p_detach = start->p_detach;
    sm.p_initial_detach = start->p_initial_detach;
    sm.p_initial_detach_decay = start->p_initial_detach_decay;
    sm.p_initial_block = start->p_initial_block;
    sm.p_cyclic_block = start->p_cyclic_block;
    for (int c = 0; c < C; c++) {
        sm.p_bleach[c] = start->p_bleach[c];
        sm.p_dud[c] = start->p_dud[c];
        sm.bg_sig[c] = start->bg_sig[c];
        sm.mu[c] = start->mu[c];
        sm.sig[c] = start->sig[c];
    }
    if (start->interactions) sm.inter.assign(start->interactions, start->interactions + C * C);
    if (start->flat_interactions) sm.flat.assign(start->flat_interactions, start->flat_interactions + C * C);

    wp_seq_model view = sm.view();
    wp_status st = wp_model_upload(ctx, &view, T);
    if (st != WP_OK) return st;
    st = wp_fit_begin(ctx, dye_seq, length, rads, R);
    if (st != WP_OK) return st;
    st = wp_fit_set_emission(ctx, fs.fit_emission ? 1 : 0);
    if (st != WP_OK) return st;

    const auto t0 = std::chrono::steady_clock::now();
    HostModel x;
    double step = 0.0;
    int iters = 0;
    while (true) {
        if (iters > 0) {
            view = sm.view();
            st = wp_model_upload(ctx, &view, T);
            if (st != WP_OK) return st;
        }
        wp_fit_sums s;
        st = wp_fit_estep(ctx, &s, nullptr, nullptr);
        if (st != WP_OK) return st;
        iters++;
        HostModel next = sm;
        {
            wp_fit_params cur = to_params(sm), nx;
            st = wp_fit_mstep(&s, C, T, dye_seq, length, (long long)R, &cur, &fs, &nx, &step);
            if (st != WP_OK) return st;
            if (fs.fit_emission) {
                wp_emission_sums es;
                st = wp_fit_emission_sums(ctx, &es);
                if (st != WP_OK) return st;
                wp_fit_params nx2;
                double estep = 0.0;
                st = wp_fit_emission_mstep(&es, C, &nx, &nx2, &estep);
                if (st != WP_OK) return st;
                nx = nx2;
                step = std::max(step, estep);
            }
            from_params(nx, &next);
        }
        const double elapsed =
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (step < stopping_threshold || elapsed > max_runtime) {
            x = next;
            break;
        }
        sm = next;
    }
    // log_likelihood(radiometries, x) (fitters/hmm-fitter.h:119-142).
    view = x.view();
    st = wp_model_upload(ctx, &view, T);
    if (st != WP_OK) return st;
    wp_fit_sums s;
    double sl = 0.0;
    int nz = 0;
    st = wp_fit_estep(ctx, &s, &sl, &nz);
    if (st != WP_OK) return st;

    out->p_edman_failure = x.p_edman_failure;
    out->p_detach = x.p_detach;
    out->p_initial_detach = x.p_initial_detach;
    out->p_initial_detach_decay = x.p_initial_detach_decay;
    out->p_initial_block = x.p_initial_block;
    out->p_cyclic_block = x.p_cyclic_block;
    for (int c = 0; c < WP_MAX_CHANNELS; c++) {
        out->p_bleach[c] = c < C ? x.p_bleach[c] : 0.0;
        out->p_dud[c] = c < C ? x.p_dud[c] : 0.0;
        out->mu[c] = c < C ? x.mu[c] : 0.0;
        out->sig[c] = c < C ? x.sig[c] : 0.0;
        out->bg_sig[c] = c < C ? x.bg_sig[c] : 0.0;
    }
    if (step_size) *step_size = step;
    if (log_l) *log_l = nz > 0 ? -INFINITY : sl;
    if (iterations) *iterations = iters;
    return WP_OK;
}

// bootstrap_fit (fitters/bootstrap-fit.cc:37-173): num_rounds fits on reads
// resampled with replacement, one fit on all reads, and per parameter the
// confidence bounds from the sorted round results.  The reference seeds its
// resampling from the clock; here the caller gives the seed (a 64-bit
// Mersenne twister draws the indices).
// B EM instances at once (the bootstrap rounds, which fitters/bootstrap-fit.
// cc:37-93 fits one after another): every iteration one batched E-step of
// the instances still running (wp_fit_estep_batch, each over its own read
// list), then each instance's M-step on the host; an instance stops as
// wp_hmm_fit does (step below the threshold or the time spent), the others
// go on.  The final log-likelihoods come from one more batched E-step with
// each instance's fitted model.
wp_status wp_hmm_fit_batch(wp_ctx* ctx, const wp_seq_model* start, int T, const int16_t* dye_seq, int length,
                           const double* rads, int R, const wp_fit_settings* settings, double stopping_threshold,
                           double max_runtime, int B, const int32_t* idx, int R_each, wp_fit_params* out_rounds,
                           double* out_log_ls, double* out_steps) {
    if (!ctx || !start || !rads || R < 1 || B < 1 || R_each < 1 || !idx || !out_rounds || !out_log_ls)
        return WP_ERR_INVALID;
    if (settings && settings->fit_emission)
        return wp_internal_fail(ctx, WP_ERR_UNSUPPORTED, "batched fits keep the emission parameters fixed");
    const int C = start->num_channels;
    if (C < 1 || C > WP_MAX_CHANNELS) return wp_internal_fail(ctx, WP_ERR_UNSUPPORTED, "num_channels out of range 1..4");
    if (!start->p_bleach || !start->p_dud || !start->bg_sig || !start->mu || !start->sig)
        return wp_internal_fail(ctx, WP_ERR_INVALID, "null per-channel array");
    wp_fit_settings fs;
    memset(&fs, 0, sizeof(fs));
    if (settings) fs = *settings;
    HostModel s0;
    s0.C = C;
    s0.p_edman_failure = start->p_edman_failure;
    s0.p_detach = start->p_detach;
    s0.p_initial_detach = start->p_initial_detach;
    s0.p_initial_detach_decay = start->p_initial_detach_decay;
    s0.p_initial_block = start->p_initial_block;
    s0.p_cyclic_block = start->p_cyclic_block;
    for (int c = 0; c < C; c++) {
        s0.p_bleach[c] = start->p_bleach[c];
        s0.p_dud[c] = start->p_dud[c];
        s0.bg_sig[c] = start->bg_sig[c];
        s0.mu[c] = start->mu[c];
        s0.sig[c] = start->sig[c];
    }
    if (start->interactions) s0.inter.assign(start->interactions, start->interactions + C * C);
    if (start->flat_interactions) s0.flat.assign(start->flat_interactions, start->flat_interactions + C * C);
    wp_seq_model v0 = s0.view();
    wp_status st = wp_model_upload(ctx, &v0, T);
    if (st != WP_OK) return st;
    st = wp_fit_begin(ctx, dye_seq, length, rads, R);
    if (st != WP_OK) return st;
    st = wp_fit_set_emission(ctx, 0);
    if (st != WP_OK) return st;

    std::vector<HostModel> cur(B, s0), fin(B, s0);
    std::vector<double> step(B, 0.0);
    std::vector<int> active(B);
    for (int b = 0; b < B; b++) active[b] = b;
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<wp_seq_model> views;
    std::vector<int32_t> lists;
    std::vector<wp_fit_sums> sums;
    while (!active.empty()) {
        const int A = (int)active.size();
        views.resize(A);
        lists.resize((size_t)A * R_each);
        sums.resize(A);
        for (int a = 0; a < A; a++) {
            views[a] = cur[active[a]].view();
            memcpy(&lists[(size_t)a * R_each], idx + (size_t)active[a] * R_each, sizeof(int32_t) * R_each);
        }
        st = wp_fit_estep_batch(ctx, views.data(), A, lists.data(), R_each, sums.data(), nullptr, nullptr);
        if (st != WP_OK) return st;
        const double elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::vector<int> still;
        for (int a = 0; a < A; a++) {
            const int b = active[a];
            wp_fit_params cp = to_params(cur[b]), nx;
            st = wp_fit_mstep(&sums[a], C, T, dye_seq, length, (long long)R_each, &cp, &fs, &nx, &step[b]);
            if (st != WP_OK) return st;
            HostModel next = cur[b];
            from_params(nx, &next);
            if (step[b] < stopping_threshold || elapsed > max_runtime) fin[b] = next;
            else {
                cur[b] = next;
                still.push_back(b);
            }
        }
        active.swap(still);
    }
    // log_likelihood of each round's fit on its reads (fitters/hmm-fitter.h:119-142)
    views.resize(B);
    sums.resize(B);
    for (int b = 0; b < B; b++) views[b] = fin[b].view();
    std::vector<double> sl(B);
    std::vector<int> nz(B);
    st = wp_fit_estep_batch(ctx, views.data(), B, idx, R_each, sums.data(), sl.data(), nz.data());
    if (st != WP_OK) return st;
    for (int b = 0; b < B; b++) {
        out_rounds[b] = to_params(fin[b]);
        for (int c = C; c < WP_MAX_CHANNELS; c++) {
            out_rounds[b].p_bleach[c] = out_rounds[b].p_dud[c] = 0.0;
            out_rounds[b].mu[c] = out_rounds[b].sig[c] = out_rounds[b].bg_sig[c] = 0.0;
        }
        out_log_ls[b] = nz[b] > 0 ? -INFINITY : sl[b];
        if (out_steps) out_steps[b] = step[b];
    }
    return WP_OK;
}

wp_status wp_hmm_bootstrap_fit(wp_ctx* ctx, const wp_seq_model* start, int T, const int16_t* dye_seq, int length,
                               const double* rads, int R, const wp_fit_settings* settings, double stopping_threshold,
                               double max_runtime, int num_rounds, double confidence_interval,
                               unsigned long long seed, wp_fit_params* out_rounds, double* out_log_ls,
                               wp_fit_params* out_best, double* out_step_size, double* out_best_log_l,
                               wp_fit_params* out_ci_min, wp_fit_params* out_ci_max,
                               double* out_worst_round_step) {
    if (!ctx || !start || !rads || R < 1 || num_rounds < 1 || !out_rounds || !out_log_ls || !out_best ||
        !(confidence_interval >= 0.0 && confidence_interval <= 1.0))
        return WP_ERR_INVALID;
    const int C = start->num_channels;
    const size_t TC = (size_t)T * C;
    std::mt19937_64 gen(seed);
    std::uniform_int_distribution<int> pick(0, R - 1);  // inclusive bounds, as the reference's
    // the rounds' resampled reads (bootstrap-fit.cc:61-70), as index lists
    std::vector<int32_t> idx((size_t)num_rounds * R);
    for (size_t i = 0; i < idx.size(); i++) idx[i] = pick(gen);
    double worst = 0.0;
    if (!(settings && settings->fit_emission)) {
        std::vector<double> steps(num_rounds);
        wp_status st = wp_hmm_fit_batch(ctx, start, T, dye_seq, length, rads, R, settings, stopping_threshold,
                                        max_runtime, num_rounds, idx.data(), R, out_rounds, out_log_ls,
                                        steps.data());
        if (st != WP_OK) return st;
        for (double x : steps) worst = std::max(worst, x);
    } else {
        // emission parameters fitted per round: the rounds' emission factors
        // differ, so they run one after another
        std::vector<double> sub((size_t)R * TC);
        for (int i = 0; i < num_rounds; i++) {
            for (int j = 0; j < R; j++)
                memcpy(&sub[(size_t)j * TC], rads + (size_t)idx[(size_t)i * R + j] * TC, sizeof(double) * TC);
            double step = 0.0;
            wp_status st = wp_hmm_fit(ctx, start, T, dye_seq, length, sub.data(), R, settings, stopping_threshold,
                                      max_runtime, &out_rounds[i], &step, &out_log_ls[i], nullptr);
            if (st != WP_OK) return st;
            worst = std::max(worst, step);
        }
    }
    double best_step = 0.0, best_ll = 0.0;
    wp_status st = wp_hmm_fit(ctx, start, T, dye_seq, length, rads, R, settings, stopping_threshold, max_runtime,
                              out_best, &best_step, &best_ll, nullptr);
    if (st != WP_OK) return st;
    if (out_step_size) *out_step_size = best_step;
    if (out_best_log_l) *out_best_log_l = best_ll;
    if (out_worst_round_step) *out_worst_round_step = worst;
    // confidence bounds per parameter (bootstrap-fit.cc:95-167); the upper
    // index is clamped to the last round (the reference reads one past the
    // end when the product is integral at confidence 1)
    const int lo = std::min(num_rounds - 1, (int)((1.0 - confidence_interval) / 2.0 * (double)num_rounds));
    const int hi = std::min(num_rounds - 1, (int)((1.0 - (1.0 - confidence_interval) / 2.0) * (double)num_rounds));
    auto bounds = [&](auto get, auto set) {
        std::vector<double> v(num_rounds);
        for (int i = 0; i < num_rounds; i++) v[i] = get(out_rounds[i]);
        std::sort(v.begin(), v.end());
        if (out_ci_min) set(*out_ci_min, v[lo]);
        if (out_ci_max) set(*out_ci_max, v[hi]);
    };
    if (out_ci_min) memset(out_ci_min, 0, sizeof(*out_ci_min));
    if (out_ci_max) memset(out_ci_max, 0, sizeof(*out_ci_max));
    bounds([](const wp_fit_params& p) { return p.p_edman_failure; }, [](wp_fit_params& p, double x) { p.p_edman_failure = x; });
    bounds([](const wp_fit_params& p) { return p.p_detach; }, [](wp_fit_params& p, double x) { p.p_detach = x; });
    bounds([](const wp_fit_params& p) { return p.p_initial_detach; }, [](wp_fit_params& p, double x) { p.p_initial_detach = x; });
    bounds([](const wp_fit_params& p) { return p.p_initial_detach_decay; },
           [](wp_fit_params& p, double x) { p.p_initial_detach_decay = x; });
    bounds([](const wp_fit_params& p) { return p.p_initial_block; }, [](wp_fit_params& p, double x) { p.p_initial_block = x; });
    bounds([](const wp_fit_params& p) { return p.p_cyclic_block; }, [](wp_fit_params& p, double x) { p.p_cyclic_block = x; });
    for (int c = 0; c < C; c++) {
        bounds([c](const wp_fit_params& p) { return p.p_bleach[c]; }, [c](wp_fit_params& p, double x) { p.p_bleach[c] = x; });
        bounds([c](const wp_fit_params& p) { return p.p_dud[c]; }, [c](wp_fit_params& p, double x) { p.p_dud[c] = x; });
        bounds([c](const wp_fit_params& p) { return p.mu[c]; }, [c](wp_fit_params& p, double x) { p.mu[c] = x; });
        bounds([c](const wp_fit_params& p) { return p.sig[c]; }, [c](wp_fit_params& p, double x) { p.sig[c] = x; });
        bounds([c](const wp_fit_params& p) { return p.bg_sig[c]; }, [c](wp_fit_params& p, double x) { p.bg_sig[c] = x; });
    }
    return WP_OK;
}

}  // extern "C"

"""Command line: `python -m whatprot_gb300 MODE [VARIANT] [OPTS...]`.

The same subcommands, flags and validation as the reference's CLI
(cc_code/src/main/main.cc:66-480): `classify hmm|hybrid|nn`, `fit`,
`simulate rad|dt`; an invalid combination prints "INCORRECT USAGE" and the
help and exits 1.  Every run prints the reference's phase lines
(main/cmd-line-out.cc) and writes the reference's file formats
(whatprot_gb300/io.py).  The work runs on the GPU through the C ABI.

Reference behaviours kept: `classify nn` builds its dye-track coordinates
with the true mu while the reads are divided by mu
(main/run-classify-nn.cc:48,76-77); `fit` takes --maxruntime in minutes.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

from . import capi, io
from .model import SequencingModel, parse_dye_seq

DBL_MAX = sys.float_info.max
INT_MAX = 2 ** 31 - 1

# (short, long, type)
OPTIONS = [("b", "numbootstrap", int), ("c", "confidenceinterval", float), ("g", "numgenerate", int),
           ("k", "neighbors", int), ("p", "hmmprune", float), ("s", "sigma", float), ("t", "timesteps", int),
           ("x", "dyeseqstring", str), ("F", "fitsettings", str), ("H", "passthrough", int),
           ("L", "stoppingthreshold", float), ("M", "maxruntime", int), ("P", "seqparams", str),
           ("R", "radiometries", str), ("S", "dyeseqs", str), ("T", "dyetracks", str), ("Y", "results", str)]

HELP = """whatprot is a program for analyzing protein fluorosequencing data.
Usage:
  whatprot [MODE] [VARIANT] [OPTS...]

  MODE is one of classify, fit, or simulate. Other parameter
  requirements depend on these.

  For MODE classify, you must define a VARIANT as one of hmm,
  hybrid, or nn.
    For VARIANT hmm, you must define --seqparams, --dyeseqs,
    --radiometries, and --results. Option --hmmprune is also
    permitted.
    For VARIANT hybrid, you must define --seqparams,
    --neighbors, --sigma, --passthrough, --dyeseqs, --dyetracks,
    --radiometries, and --results. Option --hmmprune is also
    permitted.
    For VARIANT nn, you must define --seqparams, --neighbors,
    --sigma, --dyetracks, --radiometries, and --results.

  For MODE fit, you must NOT define a VARIANT, and you MUST
  define --seqparams, --stoppingthreshold, --dyeseqstring, and
  --radiometries. You may define --fitsettings, --maxruntime (minutes),
  and BOTH --numbootstrap and --confidenceinterval (then also --results).

  For MODE simulate, you must define a VARIANT as either dt or rad.
    For VARIANT dt, you must define --seqparams, --timesteps,
    --numgenerate, --dyeseqs, and --dyetracks.
    For VARIANT rad, you must define --seqparams, --timesteps,
    --numgenerate, --dyeseqs, --radiometries, and --results

  -h, --help                    Print usage
  -b, --numbootstrap arg        bootstrap rounds (fit)
  -c, --confidenceinterval arg  confidence interval size (fit)
  -g, --numgenerate arg         reads (rad) or dye-tracks per peptide (dt)
  -k, --neighbors arg           kNN neighbours (nn, hybrid)
  -p, --hmmprune arg            HMM pruning multiplier on sigma (hmm, hybrid)
  -s, --sigma arg               Gaussian vote sigma (nn, hybrid)
  -t, --timesteps arg           timesteps (simulate)
  -x, --dyeseqstring arg        dye-seq being fitted (fit)
  -F, --fitsettings arg         JSON of held parameters (fit)
  -H, --passthrough arg         candidates from kNN to HMM (hybrid)
  -L, --stoppingthreshold arg   stopping step size (fit)
  -M, --maxruntime arg          time limit in minutes (fit)
  -P, --seqparams arg           sequencing parameters JSON
  -R, --radiometries arg        radiometries file
  -S, --dyeseqs arg             dye-seqs file
  -T, --dyetracks arg           dye-tracks file
  -Y, --results arg             predictions / true ids / bootstrap results file
"""


def parse(argv):
    """cxxopts-like: -x value, -xvalue, --long value, --long=value; unknown
    tokens are positional (the reference allows unrecognised options)."""
    by_short = {s: (l, t) for s, l, t in OPTIONS}
    by_long = {l: (l, t) for s, l, t in OPTIONS}
    opts, pos, help_ = {}, [], False
    i = 0
    while i < len(argv):
        a = argv[i]
        name, val = None, None
        if a in ("-h", "--help"):
            help_ = True
        elif a.startswith("--") and len(a) > 2:
            key = a[2:]
            if "=" in key:
                key, val = key.split("=", 1)
            if key in by_long:
                name = key
        elif a.startswith("-") and len(a) >= 2 and a[1] in by_short:
            name = a[1]
            if len(a) > 2:
                val = a[2:]
        if name is None and not (a in ("-h", "--help")):
            pos.append(a)
        elif name is not None:
            lname, typ = by_short[name] if name in by_short else by_long[name]
            if val is None:
                i += 1
                if i >= len(argv):
                    raise ValueError(f"option {a} needs a value")
                val = argv[i]
            opts[lname] = typ(val)
        i += 1
    return opts, pos, help_


def incorrect():
    print("\nINCORRECT USAGE\n")
    print(HELP)
    return 1


def _t():
    return time.perf_counter()


def _load_model(path):
    true = SequencingModel.from_json(path)
    return true, true.with_mu_as_one()


def run_classify_hmm(P, p, S, R, Y):
    t_all = _t()
    t0 = _t()
    ds = io.read_dye_seqs(S)
    print(f"Read {len(ds)} dye seqs ({_t() - t0} seconds).")
    t0 = _t()
    true, sm = _load_model(P)
    print(f"Finished basic setup ({_t() - t0} seconds).")
    t0 = _t()
    T, C, rads = io.read_radiometries(R, true)
    print(f"Read {rads.shape[0]} radiometries ({_t() - t0} seconds).")
    t0 = _t()
    clf = capi.HMMClassifier(T, C, sm, p, ds)
    print(f"Built classifier ({_t() - t0} seconds).")
    t0 = _t()
    res = clf.classify(rads) if rads.shape[0] else []
    print(f"Finished classification ({_t() - t0} seconds).")
    t0 = _t()
    io.write_predictions(Y, [r.id for r in res], [r.adjusted_score() for r in res])
    print(f"Finished saving results ({_t() - t0} seconds).")
    print(f"Total run time: {_t() - t_all} seconds.")


def run_classify_hybrid(P, k, s, H, p, S, T_, R, Y):
    t_all = _t()
    t0 = _t()
    true, sm = _load_model(P)
    print(f"Finished basic setup ({_t() - t0} seconds).")
    t0 = _t()
    ds = io.read_dye_seqs(S)
    print(f"Read {len(ds)} dye seqs ({_t() - t0} seconds).")
    t0 = _t()
    dts = io.read_dye_tracks(T_)
    print(f"Read {len(dts)} dye tracks ({_t() - t0} seconds).")
    t0 = _t()
    T, C, rads = io.read_radiometries(R, true)
    print(f"Read {rads.shape[0]} radiometries ({_t() - t0} seconds).")
    t0 = _t()
    clf = capi.HybridClassifier(T, C, sm, p, k, s, dts, H, ds)
    print(f"Built classifier ({_t() - t0} seconds).")
    t0 = _t()
    res = clf.classify(rads) if rads.shape[0] else []
    print(f"Finished classification ({_t() - t0} seconds).")
    t0 = _t()
    io.write_predictions(Y, [r.id for r in res], [r.adjusted_score() for r in res])
    print(f"Finished saving results ({_t() - t0} seconds).")
    print(f"Total run time: {_t() - t_all} seconds.")


def run_classify_nn(P, k, s, T_, R, Y):
    t_all = _t()
    t0 = _t()
    true = SequencingModel.from_json(P)
    print(f"Finished basic setup ({_t() - t0} seconds).")
    t0 = _t()
    dts = io.read_dye_tracks(T_)
    print(f"Read {len(dts)} dye tracks ({_t() - t0} seconds).")
    t0 = _t()
    T, C, rads = io.read_radiometries(R, true)
    print(f"Read {rads.shape[0]} radiometries ({_t() - t0} seconds).")
    t0 = _t()
    clf = capi.NNClassifier(T, C, true, k, s, dts)
    print(f"Built classifier ({_t() - t0} seconds).")
    t0 = _t()
    res = clf.classify(rads) if rads.shape[0] else []
    print(f"Finished classification ({_t() - t0} seconds).")
    t0 = _t()
    io.write_predictions(Y, [r.id for r in res], [r.adjusted_score() for r in res])
    print(f"Finished saving results ({_t() - t0} seconds).")
    print(f"Total run time: {_t() - t_all} seconds.")


def _fit_settings(path, C):
    """FitSettings (parameterization/settings/fit-settings.cc:44-101)."""
    holds = {}
    if not path:
        return holds
    with open(path) as f:
        data = json.load(f)
    for key in ("hold_p_edman_failure", "hold_p_detach", "hold_p_initial_detach", "hold_p_initial_detach_decay",
                "hold_p_initial_block", "hold_p_cyclic_block"):
        holds[key] = bool(data.get(key, False))
    if "channel_settings" in data:
        holds["hold_p_bleach"] = [bool(ch.get("hold_p_bleach", False)) for ch in data["channel_settings"]]
        holds["hold_p_dud"] = [bool(ch.get("hold_p_dud", False)) for ch in data["channel_settings"]]
    # extension, no reference counterpart: also fit mu, sig and bg_sig
    holds["fit_emission"] = bool(data.get("fit_emission", False))
    return holds


def _debug_string(m):
    """SequencingModel::debug_string (sequencing-model.cc:168-184)."""
    s = (f"Edman failure rate: {m.p_edman_failure:.6f}, Detach rate: {m.p_detach:.6f}, "
         f"Initial detach rate: {m.p_initial_detach:.6f}, "
         f"Initial detach decay rate: {m.p_initial_detach_decay:.6f}, "
         f"Initial blocked N-terminus rate: {m.p_initial_block:.6f}, "
         f"Cyclic blocked N-terminus rate: {m.p_cyclic_block:.6f}")
    for c, cm in enumerate(m.channel_models):
        s += f", Channel {c} info: (Bleach rate: {cm.p_bleach:.6f}, Dud rate: {cm.p_dud:.6f})"
    return s


def run_fit(L, max_runtime_s, x, P, F, R, b, c, Y):
    t_all = _t()
    t0 = _t()
    true, sm = _load_model(P)
    holds = _fit_settings(F, sm.num_channels)
    fit_emission = holds.pop("fit_emission", False)
    seq = parse_dye_seq(x)
    print(f"Finished basic setup ({_t() - t0} seconds).")
    t0 = _t()
    T, C, rads = io.read_radiometries(R, true)
    print(f"Read {rads.shape[0]} radiometries ({_t() - t0} seconds).")
    ctx = capi.Context(0)
    if c == 0.0:
        t0 = _t()
        fitted, step, log_l, _ = ctx.hmm_fit(sm, T, seq, rads, L, max_runtime_s, holds, fit_emission=fit_emission)
        print(f"Finished fitting parameters ({_t() - t0}seconds).")
    else:
        t0 = _t()
        res = ctx.bootstrap_fit(sm, T, seq, rads, L, b, c, seed=int(time.time()), max_runtime=max_runtime_s,
                                holds=holds, fit_emission=fit_emission)
        print(f"lower bounds: {_debug_string(res['ci_min'])}")
        print(f"upper bounds: {_debug_string(res['ci_max'])}")
        print(f"worst bootstrap step size: {res['worst_round_step']}")
        fitted, step, log_l = res["best"], res["step_size"], res["log_l"]
        print(f"Finished fitting parameters ({_t() - t0}seconds).")
        if Y:
            t0 = _t()
            io.write_params(Y, C, res["models"], res["log_ls"])
            print(f"Finished saving results ({_t() - t0} seconds).")
    ctx.close()
    print(f"Parameters:\n{_debug_string(fitted)}\n")
    if fit_emission:  # extension: the emission parameters, in the units of the reads divided by mu
        print(", ".join(f"Channel {c} emission: (mu: {cm.mu:.6f}, sig: {cm.sig:.6f}, bg_sig: {cm.bg_sig:.6f})"
                        for c, cm in enumerate(fitted.channel_models)) + "\n")
    print(f"log(L): {log_l:.17g}\n")
    print(f"Final step-size: {step} (under inf-norm)")
    print(f"Total run time: {_t() - t_all} seconds.")


def run_simulate_rad(t, g, P, S, R, Y):
    t_all = _t()
    t0 = _t()
    true, sm = _load_model(P)
    print(f"Finished basic setup ({_t() - t0} seconds).")
    t0 = _t()
    ds = io.read_dye_seqs(S)
    print(f"Read {len(ds)} dye seqs ({_t() - t0} seconds).")
    t0 = _t()
    ctx = capi.Context(0)
    ctx.upload_model(sm, t)
    ctx.upload_peptides(ds)
    rads, pep, _ = ctx.simulate_reads(g, seed=int(time.time() * 1e6) & 0xFFFFFFFFFFFF)
    ctx.close()
    keep = pep >= 0
    rads, ids = rads[keep], ds.ids[pep[keep]]
    print(f"Finished generating {rads.shape[0]} radiometries ({_t() - t0}seconds).")
    t0 = _t()
    io.write_radiometries(R, true, rads)
    io.write_true_ids(Y, ids)
    print(f"Finished saving results ({_t() - t0} seconds).")
    print(f"Total run time: {_t() - t_all} seconds.")


def run_simulate_dt(t, g, P, S, T_):
    t_all = _t()
    t0 = _t()
    true, sm = _load_model(P)
    print(f"Finished basic setup ({_t() - t0} seconds).")
    t0 = _t()
    ds = io.read_dye_seqs(S)
    print(f"Read {len(ds)} dye seqs ({_t() - t0} seconds).")
    t0 = _t()
    # generated and deduplicated on the device (wp_simulate_dye_tracks)
    ctx = capi.Context(0)
    ctx.upload_model(sm, t)
    ctx.upload_peptides(ds)
    ctx.timing_enable(True)
    dts = ctx.simulate_dye_track_set(g, seed=int(time.time() * 1e6) & 0xFFFFFFFFFFFF)
    gen_ms, _ = ctx.timing_read(ctx.KIND_SIM)
    dedup_ms, _ = ctx.timing_read(ctx.KIND_DEDUP)
    ctx.close()
    print(f"Finished generating {int(dts.src_hits.sum())} dye tracks ({gen_ms * 1e-3}seconds).")
    print(f"Finished deduping {len(dts)} unique dye tracks ({dedup_ms * 1e-3}seconds).")
    t0 = _t()
    io.write_dye_tracks(T_, dts)
    print(f"Finished saving results ({_t() - t0} seconds).")
    print(f"Total run time: {_t() - t_all} seconds.")


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    try:
        opts, pos, help_ = parse(argv)
    except ValueError:
        return incorrect()
    if help_:
        print(HELP)
        return 0
    n = len(opts)
    has = lambda k: k in opts  # noqa: E731
    if len(pos) < 1:
        return incorrect()
    if pos[0] == "classify":
        if len(pos) != 2:
            return incorrect()
        p = opts.get("hmmprune", DBL_MAX)
        if pos[1] == "hmm":
            if n - has("hmmprune") != 4 or not all(map(has, ("seqparams", "dyeseqs", "radiometries", "results"))):
                return incorrect()
            print(f"Using the GB300 engine ({capi.LIB_PATH}).")
            run_classify_hmm(opts["seqparams"], p, opts["dyeseqs"], opts["radiometries"], opts["results"])
            return 0
        if pos[1] == "hybrid":
            need = ("seqparams", "neighbors", "sigma", "passthrough", "dyeseqs", "dyetracks", "radiometries", "results")
            if n - has("hmmprune") != 8 or not all(map(has, need)):
                return incorrect()
            print(f"Using the GB300 engine ({capi.LIB_PATH}).")
            run_classify_hybrid(opts["seqparams"], opts["neighbors"], opts["sigma"], opts["passthrough"], p,
                                opts["dyeseqs"], opts["dyetracks"], opts["radiometries"], opts["results"])
            return 0
        if pos[1] == "nn":
            need = ("seqparams", "neighbors", "sigma", "dyetracks", "radiometries", "results")
            if n != 6 or not all(map(has, need)):
                return incorrect()
            print(f"Using the GB300 engine ({capi.LIB_PATH}).")
            run_classify_nn(opts["seqparams"], opts["neighbors"], opts["sigma"], opts["dyetracks"],
                            opts["radiometries"], opts["results"])
            return 0
        return incorrect()
    if pos[0] == "fit":
        hb, hc = has("numbootstrap"), has("confidenceinterval")
        if hb ^ hc:
            return incorrect()
        m = n
        if hb and hc:
            m -= 2
            if has("results"):
                m -= 1
        if has("fitsettings"):
            m -= 1
        if has("maxruntime"):
            m -= 1
        if len(pos) != 1 or m != 4 or not all(map(has, ("seqparams", "stoppingthreshold", "dyeseqstring",
                                                          "radiometries"))):
            return incorrect()
        print(f"Using the GB300 engine ({capi.LIB_PATH}).")
        run_fit(opts["stoppingthreshold"], 60.0 * float(opts.get("maxruntime", INT_MAX)), opts["dyeseqstring"],
                opts["seqparams"], opts.get("fitsettings", ""), opts["radiometries"], opts.get("numbootstrap", -1),
                opts.get("confidenceinterval", 0.0), opts.get("results", ""))
        return 0
    if pos[0] == "simulate":
        if len(pos) != 2:
            return incorrect()
        if pos[1] == "dt":
            need = ("seqparams", "timesteps", "numgenerate", "dyeseqs", "dyetracks")
            if n != 5 or not all(map(has, need)):
                return incorrect()
            run_simulate_dt(opts["timesteps"], opts["numgenerate"], opts["seqparams"], opts["dyeseqs"],
                            opts["dyetracks"])
            return 0
        if pos[1] == "rad":
            need = ("seqparams", "timesteps", "numgenerate", "dyeseqs", "radiometries", "results")
            if n != 6 or not all(map(has, need)):
                return incorrect()
            run_simulate_rad(opts["timesteps"], opts["numgenerate"], opts["seqparams"], opts["dyeseqs"],
                             opts["radiometries"], opts["results"])
            return 0
        return incorrect()
    return incorrect()


if __name__ == "__main__":
    sys.exit(main())

"""Sequencing model, dye-seqs and radiometries: the reference's data types.

Host-side mirror of the reference's parameterization and common types:

* ``SequencingModel`` / ``ChannelModel`` follow
  cc_code/src/parameterization/model/sequencing-model.cc:48-92 (JSON keys,
  interactions stored as ``1 - effect``), ``with_mu_as_one``
  (sequencing-model.cc:140-151, channel-model.cc:23-33), ``distance``
  (sequencing-model.cc:153-166) and the decaying detach rate
  (decaying-rate-model.cc:47-50).
* ``DyeSeq`` parsing follows cc_code/src/common/dye-seq.cc:23-58 (trailing
  '.' trimmed, '.' is -1, out-of-range reads as -1).
* ``dye_track`` follows cc_code/src/common/dye-track.cc:26-43.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from typing import List, Sequence

import numpy as np


@dataclass
class ChannelModel:
    p_bleach: float = 0.0
    p_dud: float = 0.0
    bg_sig: float = 0.0
    mu: float = 1.0
    sig: float = 0.0
    # interactions[o] multiplies mu per dye on channel o (1.0 = none);
    # flat_interactions[o] multiplies once when channel o carries any dye.
    interactions: List[float] = field(default_factory=list)
    flat_interactions: List[float] = field(default_factory=list)

    def sigma(self, amu: float) -> float:
        """channel-model.cc:35-37 -- note amu is not squared."""
        return math.sqrt(self.bg_sig * self.bg_sig + amu * self.sig * self.sig)

    def adjusted_mu(self, channel: int, counts: Sequence[int]) -> float:
        """channel-model.h:35-54."""
        amu = self.mu * float(counts[channel])
        for c, n in enumerate(counts):
            if c == channel:
                if n > 1:
                    amu *= self.flat_interactions[c]
                    amu *= self.interactions[c] ** (n - 1)
            elif n > 0:
                amu *= self.flat_interactions[c]
                amu *= self.interactions[c] ** n
        return amu


@dataclass
class SequencingModel:
    p_edman_failure: float = 0.0
    p_detach: float = 0.0
    p_initial_detach: float = 0.0
    p_initial_detach_decay: float = 0.0
    p_initial_block: float = 0.0
    p_cyclic_block: float = 0.0
    channel_models: List[ChannelModel] = field(default_factory=list)

    @property
    def num_channels(self) -> int:
        return len(self.channel_models)

    @staticmethod
    def from_json(path_or_dict) -> "SequencingModel":
        """sequencing-model.cc:48-92.  Every top-level key is required; a
        missing one raises KeyError, as nlohmann's get<double>() throws."""
        if isinstance(path_or_dict, dict):
            data = path_or_dict
        else:
            with open(path_or_dict) as f:
                data = json.load(f)
        sm = SequencingModel(
            p_edman_failure=float(data["p_edman_failure"]),
            p_detach=float(data["p_detach"]),
            p_initial_detach=float(data["p_initial_detach"]),
            p_initial_detach_decay=float(data["p_initial_detach_decay"]),
            p_initial_block=float(data["p_initial_block"]),
            p_cyclic_block=float(data["p_cyclic_block"]),
        )
        chans = data["channel_models"]
        C = len(chans)
        for cd in chans:
            cm = ChannelModel(
                p_bleach=float(cd["p_bleach"]), p_dud=float(cd["p_dud"]),
                bg_sig=float(cd["bg_sig"]), mu=float(cd["mu"]), sig=float(cd["sig"]),
                interactions=[1.0] * C, flat_interactions=[1.0] * C)
            for it in cd.get("interactions", []):
                o = int(it["other_channel"])
                if "effect" in it:
                    cm.interactions[o] = 1.0 - float(it["effect"])
                if "flat_effect" in it:
                    cm.flat_interactions[o] = 1.0 - float(it["flat_effect"])
            sm.channel_models.append(cm)
        return sm

    def to_json_dict(self) -> dict:
        chans = []
        for cm in self.channel_models:
            inter = []
            for o in range(len(cm.interactions)):
                d = {"other_channel": o}
                if cm.interactions[o] != 1.0:
                    d["effect"] = 1.0 - cm.interactions[o]
                if cm.flat_interactions[o] != 1.0:
                    d["flat_effect"] = 1.0 - cm.flat_interactions[o]
                if len(d) > 1:
                    inter.append(d)
            chans.append({"p_bleach": cm.p_bleach, "p_dud": cm.p_dud, "bg_sig": cm.bg_sig,
                          "mu": cm.mu, "sig": cm.sig, "interactions": inter})
        return {"p_edman_failure": self.p_edman_failure, "p_detach": self.p_detach,
                "p_initial_detach": self.p_initial_detach,
                "p_initial_detach_decay": self.p_initial_detach_decay,
                "p_initial_block": self.p_initial_block,
                "p_cyclic_block": self.p_cyclic_block, "channel_models": chans}

    def with_mu_as_one(self) -> "SequencingModel":
        """sequencing-model.cc:140-151 / channel-model.cc:23-33."""
        out = SequencingModel(self.p_edman_failure, self.p_detach, self.p_initial_detach,
                              self.p_initial_detach_decay, self.p_initial_block,
                              self.p_cyclic_block, [])
        for cm in self.channel_models:
            out.channel_models.append(ChannelModel(
                cm.p_bleach, cm.p_dud, cm.bg_sig / cm.mu, 1.0, cm.sig / cm.mu,
                list(cm.interactions), list(cm.flat_interactions)))
        return out

    def p_detach_at(self, t: int) -> float:
        """decaying-rate-model.cc:47-50."""
        return self.p_detach + self.p_initial_detach * math.exp(-float(t) * self.p_initial_detach_decay)

    def distance(self, other: "SequencingModel") -> float:
        """sequencing-model.cc:153-166 (channel part: channel-model.cc:39-44)."""
        d = max(abs(self.p_edman_failure - other.p_edman_failure),
                abs(self.p_detach - other.p_detach),
                abs(self.p_initial_detach - other.p_initial_detach),
                abs(self.p_initial_detach_decay - other.p_initial_detach_decay),
                abs(self.p_initial_block - other.p_initial_block),
                abs(self.p_cyclic_block - other.p_cyclic_block))
        for a, b in zip(self.channel_models, other.channel_models):
            d = max(d, abs(a.p_bleach - b.p_bleach), abs(a.p_dud - b.p_dud))
        return d

    def copy(self) -> "SequencingModel":
        return SequencingModel.from_json(self.to_json_dict())

    def has_interactions(self) -> bool:
        return any(v != 1.0 for cm in self.channel_models
                   for v in list(cm.interactions) + list(cm.flat_interactions))


def parse_dye_seq(s: str) -> np.ndarray:
    """dye-seq.cc:23-43: trailing '.' trimmed; '.' -> -1; digits -> channel."""
    s = s.rstrip(".")
    out = np.full(len(s), -1, dtype=np.int16)
    for i, ch in enumerate(s):
        if "0" <= ch <= "9":
            out[i] = ord(ch) - ord("0")
    return out


def dye_seq_string(seq: Sequence[int]) -> str:
    return "".join("." if int(d) < 0 else str(int(d)) for d in seq)


def dye_track(seq: Sequence[int], num_timesteps: int, num_channels: int) -> np.ndarray:
    """dye-track.cc:26-43: counts[t, c] = dyes of channel c at positions >= t."""
    out = np.zeros((num_timesteps, num_channels), dtype=np.int16)
    cs = np.zeros(num_channels, dtype=np.int16)
    for t in range(len(seq) - 1, -1, -1):
        d = int(seq[t])
        if d != -1:
            cs[d] += 1
        if t < num_timesteps:
            out[t] = cs
    return out


@dataclass
class DyeSeqSet:
    """Ragged dye-seqs with their ids and multiplicities (the reference's
    vector<SourcedData<DyeSeq, SourceCount<int>>>, common/sourced-data.h)."""
    num_channels: int
    seqs: List[np.ndarray]
    ids: np.ndarray
    counts: np.ndarray

    def __len__(self) -> int:
        return len(self.seqs)

    def ragged(self):
        offsets = np.zeros(len(self.seqs) + 1, dtype=np.int32)
        for i, s in enumerate(self.seqs):
            offsets[i + 1] = offsets[i] + len(s)
        flat = (np.concatenate(self.seqs).astype(np.int16) if offsets[-1] > 0
                else np.zeros(1, dtype=np.int16))
        return flat, offsets

    def max_num_dyes(self, num_timesteps: int) -> int:
        """hmm-classifier.cc:47-66."""
        dmax = 0
        for s in self.seqs:
            for c in range(self.num_channels):
                dmax = max(dmax, int(np.sum(np.asarray(s) == c)))
        return dmax

    def strings(self) -> List[str]:
        return [dye_seq_string(s) for s in self.seqs]

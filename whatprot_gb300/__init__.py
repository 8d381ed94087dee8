"""whatprot_gb300: GB300 (sm_103a) engine for whatprot's peptide-HMM
classification and fitting hot path, behind a C ABI
(include/whatprot_gb300.h).  The Python layer mirrors the reference's
classifier interface and file formats; the compute runs in CUDA kernels."""
from .model import ChannelModel, DyeSeqSet, SequencingModel, dye_track, parse_dye_seq  # noqa: F401

__all__ = ["ChannelModel", "DyeSeqSet", "SequencingModel", "dye_track", "parse_dye_seq"]

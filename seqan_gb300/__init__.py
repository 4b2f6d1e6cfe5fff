"""seqan_gb300 -- GB300-native batch pairwise alignment with SeqAn 2's call surface.

The engine is the CUDA library built from seqan_gb300/csrc (C-ABI: include/seqan_gb300.h);
this package is its host-side mirror of the reference interface.
"""
from .align import (AlignConfig, BatchOutput, ExecutionPolicy, Gaps, align_codes,  # noqa: F401
                    getCigarString, globalAlignment, globalAlignmentScore, localAlignment,
                    localAlignmentScore)
from .alphabet import decode, encode  # noqa: F401
from .scoring import BLOSUM62_AA27, Blosum62, Score  # noqa: F401
from ._native import Context, build, default_context  # noqa: F401

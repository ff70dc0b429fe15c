"""skylens_match — GB300-native descriptor matching for skylens-stream-rs.

The hot path (crates/core/src/matching.rs:144-215, ratio_match, and the
per-pair loop of crates/core/src/pipeline.rs:485-493) runs as sm_103a CUDA
kernels in libslm; this package is its Python host interface.
"""
from ._lib import SlmError, load, library_path
from .buildlib import build

# Precisions libslm implements (all bit-exact against the reference).
BUILT_PRECISIONS = ("fp32", "bf16", "fp8")
from .matching import (CAM_FRONT, CAM_LEFT, CAM_RIGHT, PAIR_CROSS, PAIR_POW2_MAX, PAIR_TEMPORAL, USIZE_MAX,
                       BatchPlan, DescriptorStore, Matcher, PairSchedule, candidate_pairs, default_matcher,
                       match_pairs, match_scheduled_pairs, ratio_match, scheduled_pairs)
from . import features, tracks

__all__ = ["SlmError", "load", "library_path", "build", "Matcher", "DescriptorStore", "BatchPlan", "PairSchedule",
           "ratio_match", "match_pairs", "match_scheduled_pairs", "candidate_pairs", "scheduled_pairs", "default_matcher",
           "PAIR_TEMPORAL", "PAIR_CROSS", "PAIR_POW2_MAX", "CAM_FRONT", "CAM_RIGHT", "CAM_LEFT", "USIZE_MAX",
           "features", "tracks"]

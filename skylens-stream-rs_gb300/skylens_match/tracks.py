"""Track building on the GPU: build_tracks with ConflictPolicy::Drop
(crates/core/src/tracks.rs:190) through libslm's C ABI.

Pairs are (image_a, image_b, matches) with matches (k, 2) of (feature of
image_a, feature of image_b); tracks come back as lists of (image, feature)
in ascending order, in first-observation order.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import SlmPair, SlmPairMatches, SlmTrackStats, check

P = ctypes.POINTER


def pack(pairs):
    """[(image_a, image_b, matches), ...] -> (slm_pair_matches array, flat (M, 2) uint32)."""
    arr = (SlmPairMatches * max(len(pairs), 1))()
    flat, first = [], 0
    for k, (a, b, m) in enumerate(pairs):
        m = np.asarray(m, dtype=np.uint32).reshape(-1, 2)
        arr[k] = SlmPairMatches(a, b, first, len(m))
        flat.append(m)
        first += len(m)
    flat = np.ascontiguousarray(np.concatenate(flat) if flat else np.zeros((0, 2), np.uint32))
    return arr, flat


def build_tracks_drop(matcher, n_features, pairs, min_length: int = 3, max_tracks: int = 100_000):
    """slm_build_tracks_drop -> (tracks, stats dict)."""
    nf = np.ascontiguousarray(n_features, dtype=np.uint32)
    arr, flat = pack(pairs)
    cap_t = max(len(flat), 1)
    cap_o = max(2 * len(flat), 1)
    toff = np.zeros(cap_t + 1, np.uint64)
    obs = np.zeros((cap_o, 2), np.uint32)
    nt, no = ctypes.c_uint64(), ctypes.c_uint64()
    st = SlmTrackStats()
    check(matcher._L.slm_build_tracks_drop(matcher.handle, nf.ctypes.data_as(P(ctypes.c_uint32)), len(nf), arr,
                                           len(pairs), flat.ctypes.data_as(P(SlmPair)), min_length, max_tracks,
                                           toff.ctypes.data_as(P(ctypes.c_uint64)), cap_t,
                                           obs.ctypes.data_as(P(SlmPair)), cap_o, ctypes.byref(nt), ctypes.byref(no),
                                           ctypes.byref(st)), "slm_build_tracks_drop")
    tracks = [[(int(i), int(f)) for i, f in obs[int(toff[t]):int(toff[t + 1])]] for t in range(nt.value)]
    return tracks, st.as_dict()

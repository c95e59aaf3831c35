"""kdigest_gb300 — GB300-native (sm_103a) batch ingest, compress and query of
t-digests, a drop-in for kdigest's GPU path (see include/kdigest_gb300.h)."""
from ._native import KdError, load as load_library  # noqa: F401
from .tdigest import (  # noqa: F401
    K0, K1, K2, K3, SCALES, Decay, GpuSession, GroupedTDigest, KeyDictionary, Server, TDigest,
    compress, default_session, merge_digests,
)

__all__ = [
    "K0", "K1", "K2", "K3", "SCALES", "Decay", "GpuSession", "GroupedTDigest", "TDigest",
    "compress", "default_session", "merge_digests", "KdError", "load_library", "Server",
    "KeyDictionary",
]

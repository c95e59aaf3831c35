"""kdigest_gb300 — GB300-native (sm_103a) batch ingest, compress and query of
t-digests, a drop-in for kdigest's GPU path (see include/kdigest_gb300.h)."""
from ._native import KdError, load as load_library  # noqa: F401
from .tdigest import (  # noqa: F401
    K0, K1, K2, K3, SCALES, Decay, GpuSession, GroupedTDigest, KeyDictionary, Server, TDigest,
    compress, default_session, gpu_cdf, gpu_cdf_many, gpu_grouped_compress_weighted,
    gpu_merge_digests, gpu_quantile, gpu_quantile_many, merge_digests,
)

__all__ = [
    "K0", "K1", "K2", "K3", "SCALES", "Decay", "GpuSession", "GroupedTDigest", "TDigest",
    "compress", "default_session", "merge_digests", "KdError", "load_library", "Server",
    "KeyDictionary", "gpu_grouped_compress_weighted", "gpu_quantile", "gpu_cdf",
    "gpu_quantile_many", "gpu_cdf_many", "gpu_merge_digests",
]

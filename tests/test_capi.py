"""Host-side checks that need no GPU: the C-ABI library loads and exports
every entry point include/kdigest_gb300.h declares; host API validation."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"KD_API\s+[\w\s\*]+?\b(kd_\w+)\s*\(", src))
    return names


def test_header_declares_entry_points():
    names = _declared()
    assert {"kd_session_create", "kd_store_ingest", "kd_store_quantile", "kd_compress",
            "kd_store_merge", "kd_store_to_bytes"} <= names


def test_library_exports_every_declared_symbol(kd):
    lib = ctypes.CDLL(os.path.join(ROOT, "kdigest_gb300", "libkdigest_gb300.so"))
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing
    from kdigest_gb300 import _native

    assert set(_native.EXPORTED) == _declared()


def test_library_reports_no_device_without_gpu(kd):
    """Without a GPU the engine refuses to create a session (no CPU fallback)."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from kdigest_gb300 import _native

    L = _native.load()
    h = ctypes.c_void_p()
    rc = L.kd_session_create(0, 0, ctypes.byref(h))
    assert rc == _native.KD_ECUDA and not h.value
    assert L.kd_status_string(rc) == b"CUDA error"


def test_decay_constructors():
    """test/test_decay.mojo:41-63."""
    from kdigest_gb300 import Decay

    assert not Decay.none().is_active()
    assert Decay.rate(0.5).is_active() and Decay.rate(0.5).rate_lambda == 0.5
    import math

    assert abs(Decay.half_life(10.0).rate_lambda - math.log(2.0) / 10.0) < 1e-12
    for h in (0.0, -1.0):
        with pytest.raises(ValueError):
            Decay.half_life(h)


def test_python_constants_match_the_header():
    """Every KD_OPT_* / KD_CLOCK_* / KD_PTR_* constant the Python side uses has
    the header's value."""
    from kdigest_gb300 import _native

    src = open(os.path.join(ROOT, "include", "kdigest_gb300.h")).read()
    defs = {m.group(1): int(m.group(2))
            for m in re.finditer(r"#define\s+(KD_(?:OPT|CLOCK|PTR)_\w+)\s+(\d+)", src)}
    used = {n: getattr(_native, n) for n in dir(_native) if re.fullmatch(r"KD_(OPT|CLOCK|PTR)_\w+", n)}
    assert used, "no constants found"
    for name, value in used.items():
        assert defs.get(name) == value, (name, value, defs.get(name))


def test_committed_tuning_record_is_applicable():
    """The committed autotuner record names every tuned parameter with a value
    from its search set, claims identical results, and applies as options."""
    from kdigest_gb300 import tune

    rec = tune.load_tuning()
    assert set(rec) == {name for name, _, _ in tune.PARAMS}
    for name, _, values in tune.PARAMS:
        assert rec[name] in values, (name, rec[name])

    class FakeSession:
        def __init__(self):
            self.calls = []

        def set_option(self, opt, value):
            self.calls.append((opt, value))

    fs = FakeSession()
    tune.apply_tuning(fs, rec)
    assert sorted(fs.calls) == sorted((opt, int(rec[name])) for name, opt, _ in tune.PARAMS)
    import json

    with open(tune.TUNING_FILE) as f:
        assert json.load(f)["results_identical"] is True


def test_library_defaults_match_the_tuning_record():
    """KdSession's built-in launch settings are the committed record's choice,
    so a session that skips the record (tuned=False) runs the same shapes."""
    from kdigest_gb300 import tune

    rec = tune.load_tuning()
    src = open(os.path.join(ROOT, "kdigest_gb300", "csrc", "kd_engine.h")).read()
    field = {"small_tile_cap": "small_cap", "large_blocks_per_sm": "large_bps",
             "small_blocks_per_sm": "small_bps", "concurrent_tiles": "concurrent_tiles"}
    for name, member in field.items():
        m = re.search(r"int\s+%s\s*=\s*(\d+);" % member, src)
        assert m and int(m.group(1)) == rec[name], (name, member)

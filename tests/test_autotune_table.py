"""The autotuner's saved table (tupan_gb300/tuning.json): its format, and
that apply_saved puts the entries of the current GPU (and only those) into
the library: split-sweep shapes per size bucket and the ensemble shape.
Host-side only (the library's tables need no device)."""

import json

import pytest

from tupan_gb300 import abi, autotune, lib
from tupan_gb300 import ensemble as en


def _lib_or_skip():
    try:
        return lib.load()
    except lib.TupanGB300Error:
        pytest.skip("CUDA library not built")


def test_shipped_table_is_well_formed():
    L = _lib_or_skip()
    nv = L.tupan_gb300_split_variants()
    with open(autotune.TABLE) as f:
        table = json.load(f)
    assert table, "no GPU in the shipped table"
    for gpu, entries in table.items():
        assert entries
        for key, e in entries.items():
            parts = key.split("|")
            if parts[0] == "ensemble":
                assert int(parts[1]) > 0
                assert e["nt"] in (128, 256) and e["prefetch"] in (0, 1)
                assert e["ib"] in (32, 64, 128, 256, 512)
            else:
                k, ni, nj = parts
                assert k in abi.SIGNATURES, key
                assert int(ni) > 0 and int(nj) > 0
                assert 0 <= e["variant"] < nv and e["gsplit"] >= 1, key
            assert e["seconds"] > 0


def _write(tmp_path, table):
    p = tmp_path / "tuning.json"
    p.write_text(json.dumps(table))
    return str(p)


def test_apply_saved_takes_this_gpus_entries(tmp_path, monkeypatch):
    _lib_or_skip()
    path = _write(tmp_path, {
        "Fake GPU": {
            "acc_jerk_kernel|1024|65536": {"variant": 4, "gsplit": 8,
                                           "seconds": 1e-4},
            "ensemble|64": {"nt": 128, "ib": 32, "prefetch": 0,
                            "seconds": 0.1},
            "ensemble|4096": {"nt": 256, "ib": 64, "prefetch": 1,
                              "seconds": 0.5}},
        "Other GPU": {
            "ensemble|8192": {"nt": 128, "ib": 512, "prefetch": 1,
                              "seconds": 0.5}}})
    monkeypatch.setattr(autotune, "_device_name", lambda: "Fake GPU")
    old = en.default_shape()
    try:
        assert autotune.apply_saved(path) == 3
        # the entry measured on the most systems sets the default
        assert en.default_shape() == (256, 64, 1)
    finally:
        en.set_default_shape(*old)


def test_apply_saved_without_entries_changes_nothing(tmp_path, monkeypatch):
    _lib_or_skip()
    path = _write(tmp_path, {"Other GPU": {
        "ensemble|4096": {"nt": 256, "ib": 512, "prefetch": 1,
                          "seconds": 0.5}}})
    monkeypatch.setattr(autotune, "_device_name", lambda: "Fake GPU")
    old = en.default_shape()
    assert autotune.apply_saved(path) == 0
    assert en.default_shape() == old
    assert autotune.apply_saved(str(tmp_path / "absent.json")) == 0


def test_apply_saved_rejects_a_bad_entry(tmp_path, monkeypatch):
    _lib_or_skip()
    path = _write(tmp_path, {"Fake GPU": {
        "acc_jerk_kernel|1024|65536": {"variant": 999, "gsplit": 1,
                                       "seconds": 1e-4}}})
    monkeypatch.setattr(autotune, "_device_name", lambda: "Fake GPU")
    with pytest.raises(lib.TupanGB300Error):
        autotune.apply_saved(path)


def test_library_load_applies_no_table_without_a_device(monkeypatch):
    # in a process without a GPU the device name is unknown: nothing to apply
    _lib_or_skip()
    if lib.device_name() is not None:
        pytest.skip("a GPU is present")
    assert lib.device_name() is None


def test_centred_mid_reach_setter():
    _lib_or_skip()
    prev = lib.set_centred_mid(2.0)
    try:
        assert lib.set_centred_mid(0.0) == 2.0
        for bad in (-1.0, 65.0, float("nan")):
            with pytest.raises(lib.TupanGB300Error):
                lib.set_centred_mid(bad)
        assert lib.set_centred_mid(0.0) == 0.0
    finally:
        lib.set_centred_mid(prev)


def test_ensemble_default_shape_rejects_bad_shapes():
    _lib_or_skip()
    from tupan_gb300 import ensemble as en
    old = en.default_shape()
    try:
        for bad in ((64, 128, 1), (128, 96, 1), (128, 128, 2), (512, 128, 0),
                    (128, 1024, 0)):
            with pytest.raises(lib.TupanGB300Error):
                en.set_default_shape(*bad)
        assert en.default_shape() == old
        en.set_default_shape(256, 32, 1)
        assert en.default_shape() == (256, 32, 1)
    finally:
        en.set_default_shape(*old)


def test_apply_saved_lenient_skips_a_bad_entry(tmp_path, monkeypatch):
    # what the library's load does: a stale entry is skipped with a warning
    _lib_or_skip()
    path = _write(tmp_path, {"Fake GPU": {
        "acc_jerk_kernel|1024|65536": {"variant": 999, "gsplit": 1,
                                       "seconds": 1e-4},
        "acc_kernel|1024|65536": {"variant": 4, "gsplit": 8,
                                  "seconds": 1e-4}}})
    monkeypatch.setattr(autotune, "_device_name", lambda: "Fake GPU")
    with pytest.warns(UserWarning):
        assert autotune.apply_saved(path, strict=False) == 1

"""CPU: bench.py reports a committed ncu profile only for the kernel it times.

The sweep's roofline carries DRAM traffic and the texture pipe's share from
profiles/traffic.json.  Those figures apply only while the digest of the
kernel sources and of the build recipe (its compiler flags) matches, and
only to the form they were taken on (storage, interpolation, launch form,
coarse-to-fine and exploration schedule).
"""
import argparse
import importlib.util
import json
import os
import shutil

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def chosen_args(**kw):
    d = dict(fp16=True, interp=1, per_view=False, coarse=2, exploration=3)
    d.update(kw)
    return argparse.Namespace(**d)


def stored():
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
        return json.load(f)["k_plane_sweep"]["c2"]


def test_digest_covers_sources_and_build_recipe(bench, tmp_path, monkeypatch):
    pkg = tmp_path / "recon-scanner_gb300"
    (pkg / "csrc").mkdir(parents=True)
    for name in bench.KERNEL_SOURCES:
        shutil.copy(os.path.join(ROOT, "recon-scanner_gb300", "csrc", name), pkg / "csrc" / name)
    shutil.copy(os.path.join(ROOT, "recon-scanner_gb300", "build.py"), pkg / "build.py")
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    d0 = bench.kernel_sources_digest()
    assert len(d0) == 16 and int(d0, 16) >= 0
    with open(pkg / "build.py", "a") as f:
        f.write("\n# another flag\n")
    d1 = bench.kernel_sources_digest()
    assert d1 != d0
    with open(pkg / "csrc" / bench.KERNEL_SOURCES[0], "a") as f:
        f.write("\n// another line\n")
    assert bench.kernel_sources_digest() not in (d0, d1)


def test_profile_applies_only_to_its_sources_and_form(bench, monkeypatch):
    prof = stored()
    monkeypatch.setattr(bench, "kernel_sources_digest", lambda: prof["sources_digest"])
    assert bench.sweep_profile("c2", chosen_args())["applies"] is True
    for kw in (dict(exploration=0), dict(coarse=0), dict(interp=0), dict(fp16=False), dict(per_view=True)):
        out = bench.sweep_profile("c2", chosen_args(**kw))
        assert out["applies"] is False and "form" in out["why"], kw
    monkeypatch.setattr(bench, "kernel_sources_digest", lambda: "0" * 16)
    out = bench.sweep_profile("c2", chosen_args())
    assert out["applies"] is False and "sources" in out["why"]
    assert bench.sweep_profile("c9", chosen_args())["applies"] is False

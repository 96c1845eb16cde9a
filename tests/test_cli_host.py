"""The module CLI's host-only parts: JSON ledgers (stitch, check) and config
errors, without a GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "isosurface-analysis_gb300")
CLI = os.path.join(PKG, "bin", "isosim")


@pytest.fixture(scope="module")
def cli():
    if not os.path.exists(CLI):
        subprocess.run([sys.executable, os.path.join(PKG, "build.py")], check=True)
    return CLI


def ledger(variables, volumes, maps):
    return {"dimensions": [8, 8, 8], "variables": variables, "dfDownscale": 1,
            "volumes": [{"variable": v, "timestep": t, "numIsovalues": 3, "runtime": 1.5,
                         "representatives": [{"valueId": 2, "isovalue": 0.5, "repId": 0, "importance": 2.0,
                                              "filename": "x.dat", "mapId": 1}]} for v, t in volumes],
            "similarityMaps": [{"var1": a, "t1": t1, "var2": b, "t2": t2, "filename": f} for a, t1, b, t2, f in maps]}


def test_stitch_merges_ledgers(cli, tmp_path):
    host = ledger(["A"], [(0, 1)], [(0, 1, 0, 1, "a.dat")])
    part = ledger(["B", "A"], [(0, 2), (1, 3)], [(0, 2, 1, 2, "ba.dat")])
    (tmp_path / "host.json").write_text(json.dumps(host))
    (tmp_path / "part.json").write_text(json.dumps(part))
    r = subprocess.run([cli, "stitch", "host.json", "part.json"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = json.loads((tmp_path / "stitched.json").read_text())
    assert out["variables"] == ["A", "B"]
    assert [(v["variable"], v["timestep"]) for v in out["volumes"]] == [(0, 1), (1, 2), (0, 3)]
    assert [(m["var1"], m["t1"], m["var2"], m["t2"]) for m in out["similarityMaps"]] == [(0, 1, 0, 1), (1, 2, 0, 2)]
    assert list(out.keys()) == ["dimensions", "variables", "dfDownscale", "volumes", "similarityMaps"]
    rep = out["volumes"][0]["representatives"][0]
    assert list(rep.keys()) == ["valueId", "isovalue", "repId", "importance", "filename", "mapId"]


def test_check_lists_missing_maps(cli, tmp_path):
    led = ledger(["A", "B"], [], [(0, 0, 1, 0, "x"), (0, 0, 0, 1, "y")])
    (tmp_path / "meta.json").write_text(json.dumps(led))
    r = subprocess.run([cli, "check", "meta.json", "0", "2"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 2
    assert "Missing A B 1 1" in r.stdout and "Missing B B 0 1" in r.stdout and "2 missing" in r.stdout


def test_malformed_config_is_an_error(cli, tmp_path):
    # the reference ships one config with a missing comma (configs/ionization-distance-ALL.json)
    (tmp_path / "bad.json").write_text('{"entries": [{"outputFolder": "o/" "jsonFile": "m.json"}]}')
    r = subprocess.run([cli, "script", "bad.json"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 2 and "json" in r.stderr

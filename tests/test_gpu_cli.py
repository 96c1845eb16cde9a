"""The module CLI end to end on the GPU: single (voxel approximation), script
(marching cubes) and multi (cross maps), against the engine API and the oracle."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "isosurface-analysis_gb300", "bin", "isosim")


def write_dat(path, vol):
    # .dat files are x-fastest: element x + y*X + z*X*Y
    np.asarray(vol, np.float32).transpose(2, 1, 0).tofile(path)


def make_volume(seed, dims=(20, 18, 16)):
    import isosim.synth as synth
    return synth.gaussian_blobs(dims, 4, seed, sigma=(2.0, 5.0))


def test_single_module(tmp_path):
    import isosim
    dims = (20, 18, 16)
    vol = make_volume(1, dims)
    write_dat(tmp_path / "vol.dat", vol)
    cfg = {"fileName": str(tmp_path / "vol"), "dimensions": list(dims), "minValue": -1e9, "maxValue": 1e9,
           "outputFolder": str(tmp_path / "out"), "variableName": "V", "timestep": 3, "jsonFile": "meta.json",
           "dfDownscale": 1, "engine": {"isovalues": 24, "bins": 32, "representatives": 5}}
    (tmp_path / "single.json").write_text(json.dumps(cfg))
    r = subprocess.run([CLI, "single", str(tmp_path / "single.json")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    lo, hi = oracle.real_range(vol, -1e9, 1e9)
    isos = oracle.isovalues(vol, lo, hi, 24, uniform=True)
    with isosim.Context(0) as ctx:
        # map.dat holds the reference's own FP32 map (the module default)
        ctx.set_mi_mode(isosim.MI_REF32)
        ism, ids, _, _ = ctx.ism(vol.ravel(), dims, isos, surface=isosim.SURFACE_APPROX, bins=32)
    folder = tmp_path / "out" / "V-3"
    got = np.fromfile(folder / "similarityMap-24--approx-scale_1" / "map.dat", np.float32)
    assert np.array_equal(got, ism.ravel())
    reps = isosim.select_representatives(ism, ids, isos, 5)
    meta = json.loads((tmp_path / "out" / "meta.json").read_text())
    vol_info = meta["volumes"][0]
    assert meta["variables"] == ["V"] and vol_info["timestep"] == 3 and vol_info["numIsovalues"] == len(ids)
    assert [r["valueId"] for r in vol_info["representatives"]] == [r[2] for r in reps]
    rank = sorted(r[2] for r in reps)
    for r in reps:
        df = np.fromfile(folder / "distancefields" / ("distancefield-%d.df" % rank.index(r[2])), np.float32)
        cells = oracle.approximation(vol, dims, float(isos[r[2]])).astype(np.float32)
        assert np.array_equal(df, oracle.distance_field_f32(oracle.normalize_points(cells, dims), dims))
    # a second run skips the processed volume
    r = subprocess.run([CLI, "single", str(tmp_path / "single.json")], capture_output=True, text=True)
    assert "already processed" in r.stdout
    assert len(json.loads((tmp_path / "out" / "meta.json").read_text())["volumes"]) == 1


def test_script_then_multi(tmp_path):
    import isosim
    dims = (16, 16, 16)
    variables = ["A", "B"]
    steps = [0, 1]
    inp = tmp_path / "in"
    for v in variables:
        (inp / v).mkdir(parents=True)
        for t in steps:
            write_dat(inp / v / ("%s%04d.dat" % (v, t)), make_volume(10 * len(v) + t + (5 if v == "B" else 0), dims))
    cfg = {"entries": [{"dimensions": list(dims), "timesteps": steps, "dfDownscale": 1,
                        "fileFormatString": "%s/%s/%s%04d", "inputFolder": str(inp),
                        "outputFolder": str(tmp_path / "out"), "jsonFile": "meta.json",
                        "variables": [{"name": v, "minValue": -1e9, "maxValue": 1e9, "variableFolder": v}
                                      for v in variables],
                        "engine": {"isovalues": 40, "bins": 32}}]}
    (tmp_path / "script.json").write_text(json.dumps(cfg))
    r = subprocess.run([CLI, "script", str(tmp_path / "script.json")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    meta = json.loads((tmp_path / "out" / "meta.json").read_text())
    assert len(meta["volumes"]) == 4 and all(len(v["representatives"]) == 16 for v in meta["volumes"])
    mcfg = {"jsonFile": "meta.json", "timeSteps": steps, "dataRoot": str(tmp_path / "out"), "dfDownscale": 1,
            "engine": {"bins": 32}}
    (tmp_path / "multi.json").write_text(json.dumps(mcfg))
    r = subprocess.run([CLI, "multi", str(tmp_path / "multi.json")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    meta = json.loads((tmp_path / "out" / "meta.json").read_text())
    names = meta["variables"]
    cross = [(names[m["var1"]], m["t1"], names[m["var2"]], m["t2"], m["filename"]) for m in meta["similarityMaps"]
             if m["filename"].endswith(".dat") and "TMP-multiMap" in m["filename"]]
    assert sorted((a, t1, b, t2) for a, t1, b, t2, _ in cross) == [("A", 0, "A", 1), ("A", 0, "B", 0),
                                                                   ("A", 1, "B", 1), ("B", 0, "B", 1)]
    F = 16 ** 3
    for a, t1, b, t2, f in cross:
        got = np.fromfile(f, np.float32).reshape(16, 16)
        fa = [np.fromfile(tmp_path / "out" / ("%s-%d" % (a, t1)) / "distancefields" / ("distancefield-%d.df" % i),
                          np.float32) for i in range(16)]
        fb = [np.fromfile(tmp_path / "out" / ("%s-%d" % (b, t2)) / "distancefields" / ("distancefield-%d.df" % i),
                          np.float32) for i in range(16)]
        for i in range(16):
            for j in range(16):
                joint, cs, rs = oracle.pair_histogram(fa[i], fb[j], 32, oracle.field_interval(fa[i]),
                                                      oracle.field_interval(fb[j]))
                # the reference's FP32 MI (device evaluation vs the host restatement)
                assert abs(got[i, j] - oracle.mi_f32(joint, cs, rs, F)) < 1e-5
    r = subprocess.run([CLI, "check", str(tmp_path / "out" / "meta.json"), "0", "2"], capture_output=True, text=True)
    assert r.returncode == 0 and "0 missing" in r.stdout
    # timestep and variable similarity matrices over those cross maps
    agg = {(a["kind"], a["variable"], a["timestep"]): a["filename"] for a in meta["aggregateMaps"]}
    assert set(agg) == {("TSM", 0, -1), ("TSM", 1, -1), ("VSM", -1, 0), ("VSM", -1, 1)}
    maps = {(a, t1, b, t2): np.fromfile(f, np.float32).reshape(16, 16) for a, t1, b, t2, f in cross}

    def summary(m):
        return float(m.mean()), 0.5 * (float(m.max(axis=1).mean()) + float(m.max(axis=0).mean()))

    tsm = json.loads(open(agg[("TSM", names.index("A"), -1)]).read())
    assert tsm["variable"] == "A" and tsm["timesteps"] == steps
    mean, best = summary(maps[("A", 0, "A", 1)])
    assert abs(tsm["mean"][0][1] - mean) < 1e-5 and abs(tsm["bestMatch"][0][1] - best) < 1e-5
    assert abs(tsm["bestMatch"][1][0] - best) < 1e-5 and tsm["mean"][0][0] == 1.0
    vsm = json.loads(open(agg[("VSM", -1, 1)]).read())
    assert vsm["variables"] == names
    mean, best = summary(maps[("A", 1, "B", 1)])
    ia, ib = names.index("A"), names.index("B")
    assert abs(vsm["mean"][ia][ib] - mean) < 1e-5 and abs(vsm["bestMatch"][ia][ib] - best) < 1e-5


def test_short_volume_file_is_an_error(tmp_path):
    """A .dat file with fewer than X*Y*Z floats: the module stops with an
    error naming the file, and writes no map."""
    dims = (20, 18, 16)
    vol = make_volume(2, dims)
    write_dat(tmp_path / "vol.dat", vol)
    data = (tmp_path / "vol.dat").read_bytes()
    (tmp_path / "vol.dat").write_bytes(data[: len(data) - 4 * 17])
    cfg = {"fileName": str(tmp_path / "vol"), "dimensions": list(dims), "minValue": -1e9, "maxValue": 1e9,
           "outputFolder": str(tmp_path / "out"), "variableName": "V", "timestep": 0, "jsonFile": "meta.json",
           "dfDownscale": 1, "engine": {"isovalues": 8, "bins": 32}}
    (tmp_path / "single.json").write_text(json.dumps(cfg))
    r = subprocess.run([CLI, "single", str(tmp_path / "single.json")], capture_output=True, text=True)
    assert r.returncode != 0
    assert "short read" in r.stderr and "vol.dat" in r.stderr
    assert not (tmp_path / "out" / "meta.json").exists()


def test_allocation_failure_leaves_context_usable():
    """An allocation the context may not make (its byte cap) fails the call
    with ISO_ERR_NOMEM; the same context then runs the request normally."""
    import isosim
    vol = make_volume(3, (32, 32, 32))
    import isosim.synth as synth
    isos = synth.inside_isovalues(vol, 12)
    with isosim.Context(0) as ref:
        want, want_ids, _, _ = ref.ism(vol.ravel(), (32, 32, 32), isos, bins=64)
    with isosim.Context(0) as ctx:
        ctx.set_device_bytes_cap(1 << 20)
        with pytest.raises(isosim.IsoError) as e:
            ctx.ism(vol.ravel(), (32, 32, 32), isos, bins=64)
        assert e.value.code == isosim.ISO_ERR_NOMEM and "cap" in str(e.value)
        assert ctx.device_bytes <= 1 << 20
        ctx.set_device_bytes_cap(0)
        got, ids, _, _ = ctx.ism(vol.ravel(), (32, 32, 32), isos, bins=64)
    assert np.array_equal(ids, want_ids) and np.array_equal(got, want)

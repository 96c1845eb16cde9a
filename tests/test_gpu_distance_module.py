"""The distance module (isovalue equalisation) end to end on the GPU.

The CLI's isovalues, iteration by iteration, are checked against a separate
float32 restatement of the reference's default-path algorithm
(DistanceEqualization.cpp: approximation :84-131, evaluateDistances :333-557,
binaryIsoValueSearch :1338-1449, binarySearchEqualization :1451-1619) that
measures each candidate set with the engine's own similarity map."""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "isosurface-analysis_gb300", "bin", "isosim")
ND, MAX_ITR, STEP_ITR = 16, 180, 5
f32 = np.float32


def write_dat(path, vol):
    np.asarray(vol, np.float32).transpose(2, 1, 0).tofile(path)


class Restated:
    def __init__(self, ctx, vol, dims, vmin, vmax, bins):
        self.ctx, self.vol, self.dims, self.bins = ctx, vol.ravel(), dims, bins
        self.vmin, self.vmax = f32(vmin), f32(vmax)
        self.fixed = [True] + [False] * (ND - 1) + [True]
        self.best_avg, self.best = f32(10e20), None
        self.moving = [[f32(0), f32(0)] for _ in range(ND)]
        self.infos = []
        self.rows = []

    def count(self, iso):
        import isosim
        pts, _ = self.ctx.surface_points(self.vol, self.dims, [iso], surface=isosim.SURFACE_APPROX)
        return len(pts[0])

    def measure(self, iso):
        import isosim
        for d in range(ND + 1):
            n = self.count(iso[d])
            cur = iso[d]
            val = iso[d + 1] if d < ND else f32(cur + f32((self.vmax - self.vmin) / f32(ND)))
            incr = f32((val - cur) / f32(ND))
            while n == 0:
                cur = f32(cur + incr)
                if cur > self.vmax or cur != cur:
                    cur = iso[d - 1] if d > 0 else self.vmin
                    incr = f32((iso[d] - cur) / f32(16))
                    cur = f32(cur + incr)
                if d < ND and cur > iso[d + 1]:
                    iso[d] = iso[d + 1]
                    iso[d + 1] = cur
                    cur = iso[d]
                iso[d] = cur
                n = self.count(cur)
        ism, ids, _, _ = self.ctx.ism(self.vol, self.dims, np.array(iso, np.float32),
                                      surface=isosim.SURFACE_APPROX, bins=self.bins)
        assert len(ids) == ND + 1
        self.dist = [f32(f32(1) - ism[j, j + 1]) for j in range(ND)]

    def evaluate(self, iso, fix_even):
        acc = f32(0)
        for d in self.dist:
            acc = f32(acc + d)
        avg = f32(acc / f32(ND))
        err = f32(0)
        for d in self.dist:
            err = f32(err + f32(abs(f32(d - avg))))
        avg_e = f32(err / f32(ND))
        if f32(avg_e / avg) < self.best_avg:
            self.best_avg = f32(avg_e / avg)
            self.best = list(iso)
        for i in range(1 if fix_even else 0, ND - 1, 2):
            if i == 0:
                continue
            dl, dr = self.dist[i - 1], self.dist[i]
            if abs(f32(dl - dr)) < abs(f32(self.moving[i - 1][0] - self.moving[i][0])):
                self.moving[i - 1] = [dl, iso[i - 1]]
                self.moving[i] = [dr, iso[i]]

    def move(self, fixed_even, it, iso, info):
        for i in range(1 if fixed_even else 2, ND, 2):
            j, k = i - 1, i + 1
            dji, dik = self.dist[j], self.dist[i]
            s = f32(dji + dik)
            if it % STEP_ITR == 0:
                up, lo = (iso[k], s, f32(0)), (iso[j], f32(0), s)
            else:
                up, lo = self.infos[it - 1]["up"][i], self.infos[it - 1]["lo"][i]
            if dji > dik:
                up = (iso[i], dji, dik)
            if dji < dik:
                lo = (iso[i], dji, dik)
            with np.errstate(all="ignore"):
                i1 = f32(f32(lo[1] - up[1]) / f32(lo[0] - up[0]))
                x1 = f32(lo[1] - f32(i1 * lo[0]))
                i2 = f32(f32(lo[2] - up[2]) / f32(lo[0] - up[0]))
                x2 = f32(lo[2] - f32(i2 * lo[0]))
                nv = f32(f32(x2 - x1) / f32(i1 - i2))
            if not np.isnan(nv) and not self.fixed[i]:
                iso[i] = nv
            info["up"][i], info["lo"][i] = up, lo

    def fix_inversions(self, iso):
        for i in range(ND + 1):
            for j in range(i + 1, ND + 1):
                if iso[i] > iso[j]:
                    iso[i], iso[j] = iso[j], iso[i]
                    self.fixed[i], self.fixed[j] = self.fixed[j], self.fixed[i]

    def run(self, start):
        iso = list(start)
        self.measure(iso)
        self.evaluate(iso, False)
        self.rows.append(list(iso))
        cur = list(self.best)
        self.moving = [[self.dist[j], self.best[j]] for j in range(ND)]
        fixed_even = True
        for it in range(MAX_ITR + 1):
            if it > 0:
                cur = list(self.infos[-1]["iso"])
            self.fix_inversions(cur)
            info = {"up": {}, "lo": {}}
            self.move(fixed_even, it, cur, info)
            self.measure(cur)
            self.evaluate(cur, fixed_even)
            info["iso"] = list(cur)
            self.infos.append(info)
            self.rows.append(list(cur))
            if (it + 1) % STEP_ITR == 0:
                self.dist = [self.moving[i][0] for i in range(ND)]
                fixed_even = not fixed_even


def test_distance_module_matches_restatement(tmp_path):
    import isosim
    import isosim.synth as synth
    dims = (24, 22, 20)
    vol = synth.gaussian_blobs(dims, 5, 31, sigma=(2.5, 6.0))
    write_dat(tmp_path / "vol.dat", vol)
    cfg = {"fileName": str(tmp_path / "vol"), "dimensions": list(dims), "minValue": -1e9, "maxValue": 1e9,
           "outputFolder": str(tmp_path / "out"), "variableName": "V", "timestep": 2, "jsonFile": "meta.json",
           "dfDownscale": 1, "engine": {"bins": 32}}
    (tmp_path / "d.json").write_text(json.dumps(cfg))
    r = subprocess.run([CLI, "distance", str(tmp_path / "d.json")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    folder = tmp_path / "out" / "V-2"
    lines = (folder / "isovalues.csv").read_text().strip().splitlines()
    assert lines[0].startswith("iterations,iv0") and lines[1].startswith("estimate,")
    assert lines[-1].startswith("final,") and len(lines) == 2 + MAX_ITR + 1
    got = [np.array([float(x) for x in ln.split(",")[1:ND + 2]], np.float32) for ln in lines[1:]]

    with isosim.Context(0) as ctx:
        ctx.set_mi_mode(isosim.MI_REF32)
        vmin, vmax = ctx.real_range(vol.ravel(), -1e9, 1e9)
        rs = Restated(ctx, vol, dims, vmin, vmax, 32)
        step = f32(f32(f32(vmax) - f32(vmin)) / f32(ND))
        rs.run([f32(f32(vmin) + f32(step * f32(i))) for i in range(ND + 1)])
    assert len(rs.rows) == len(got)
    for k, (a, b) in enumerate(zip(got, rs.rows)):
        assert np.array_equal(a, np.array(b, np.float32)), k

    meta = json.loads((tmp_path / "out" / "meta.json").read_text())
    names = meta["variables"]
    assert names == ["V-%f" % 0.66]
    assert [v["runtime"] for v in meta["volumes"]] == [float(i) for i in range(0, MAX_ITR + 1, 10)]
    assert all(v["numIsovalues"] == 17 and len(v["representatives"]) == 17 for v in meta["volumes"])
    dist = [ln.split(",") for ln in (folder / "distances.csv").read_text().strip().splitlines()[1:]]
    norm_avg = [float(d[-1]) for d in dist]
    assert min(norm_avg) < norm_avg[0]  # the refinement found a more even set than the start
    # a second run of the same timestep is skipped
    r = subprocess.run([CLI, "distance", str(tmp_path / "d.json")], capture_output=True, text=True)
    assert "already processed" in r.stdout

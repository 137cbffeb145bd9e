"""GPU engine parity: the CUDA path through the C ABI against the reference's
recorded outputs (tests/golden) and the FP64 oracle.

Tolerances (the engine computes per-sample work in FP32, reductions
compensated, the normal-equation solve in FP64):
  * interpolated values: |d| <= 2e-6 x full scale (255 or 65535);
  * objectives (FP64 path): 1e-12 relative;
  * searches: status identical; u, v, w within 1e-3 voxel; objmin within
    1e-5 relative (converged points), rotation/strain within 1e-3.
"""
import numpy as np
import pytest

from fixtures import (SHAPE, case_params, hotpath, interp_params, planar_flag, search_cases,
                      strain_cases, strain_flags)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(gpu_lib):
    from digitalvolumecorrelation_gb300 import engine
    return engine


@pytest.mark.parametrize("vs", ["A", "B"])
@pytest.mark.parametrize("it", [0, 1, 2])
def test_interpolation_vs_reference(eng, vs, it):
    d = hotpath()
    p = interp_params(vs)
    E = eng.Engine(p, d[f"vol_{vs}_ref"], d[f"vol_{vs}_cor"])
    got = E.interpolate(1, d[f"interp_{vs}_{it}_center"], d[f"interp_{vs}_{it}_pts"], it)
    ref = d[f"interp_{vs}_{it}_val"]
    full = 255.0 if vs == "A" else 65535.0
    assert np.max(np.abs(got - ref)) <= 2e-6 * full
    E.close()


def test_interpolation_range_fail(eng):
    d = hotpath()
    p = interp_params("A")
    E = eng.Engine(p, d["vol_A_ref"], d["vol_A_cor"])
    c = np.array([20.0, 20.0, 20.0])
    assert E.interpolate(1, c, np.array([[c[0] + 9.6, 20.0, 20.0]]), 2) is None
    assert E.interpolate(1, c, np.array([[c[0] + 9.4, 20.0, 20.0]]), 2) is not None


@pytest.mark.parametrize("fcn", range(5))
def test_objective_vs_reference(eng, fcn):
    d = hotpath()
    o, res = eng.objective(fcn, d["obj_ref"], d["obj_tar"], residual=True)
    np.testing.assert_allclose(o, d[f"obj_{fcn}_val"][0], rtol=1e-12)
    # residuals of centred values cancel: tolerance relative to the input scale
    scale = max(np.abs(d["obj_ref"]).max(), np.abs(d["obj_tar"]).max())
    np.testing.assert_allclose(res, d[f"obj_{fcn}_res"], rtol=1e-12, atol=1e-14 * scale)


@pytest.mark.parametrize("k", range(8))
def test_search_vs_reference(eng, k):
    d = hotpath()
    case = search_cases()[k]
    p = case_params(case)
    vs = case["volumes"]
    E = eng.Engine(p, d[f"vol_{vs}_ref"], d[f"vol_{vs}_cor"])
    r = E.process(d["search_points"], order=d["search_order"], neigh=d["search_neigh"])
    st = d[f"search_{k}_status"]
    np.testing.assert_array_equal(r["status"], st)
    good = st == 0
    du = np.abs(r["params"][good, :3] - d[f"search_{k}_params"][good, :3])
    assert du.max() <= 1e-3, du.max()
    ndof = case["num_srch_dof"]
    if ndof > 3:
        dr = np.abs(r["params"][good, 3:ndof] - d[f"search_{k}_params"][good, 3:ndof])
        assert dr.max() <= 1e-3, dr.max()
    ro = d[f"search_{k}_objmin"][good]
    rel = np.abs(r["objmin"][good] - ro) / np.maximum(np.abs(ro), 1e-300)
    assert rel.max() <= 1e-5, rel.max()
    E.close()


@pytest.mark.parametrize("cluster", [1, 2, 8])
@pytest.mark.parametrize("k", [1, 6])
def test_search_cluster_sizes(eng, k, cluster, monkeypatch):
    """Every cluster width (CTAs cooperating on one point) gives the same answers."""
    monkeypatch.setenv("DVC_CLUSTER", str(cluster))
    d = hotpath()
    case = search_cases()[k]
    vs = case["volumes"]
    E = eng.Engine(case_params(case), d[f"vol_{vs}_ref"], d[f"vol_{vs}_cor"])
    r = E.process(d["search_points"], order=d["search_order"], neigh=d["search_neigh"])
    np.testing.assert_array_equal(r["status"], d[f"search_{k}_status"])
    good = r["status"] == 0
    assert np.abs(r["params"][good, :3] - d[f"search_{k}_params"][good, :3]).max() <= 1e-3
    E.close()


@pytest.mark.parametrize("name", ["vol", "vol_t", "planar"])
def test_strain_vs_reference(eng, name):
    c = strain_cases()[name]
    ndp, objt, refill = strain_flags(c["args"])
    pts = c["points"]
    out = eng.strain(pts, c["status"], c["objmin"], c["disp"], c["neigh"], ndp=ndp, objt=objt,
                     refill=refill, planar=planar_flag(pts))
    L, E, D = c["Lstr"], c["Estr"], c["dgrd"]
    np.testing.assert_array_equal(out["pts_in_sw"], L[:, 7].astype(int))
    for got, printed in ((out["u_fit"], L[:, 4:7]), (out["sw_radius"], L[:, 8]),
                         (out["l_strain"], L[:, 9:18]), (out["e_strain"], E[:, 9:18]),
                         (out["dgrad"], D[:, 9:18])):
        printed = np.asarray(printed)
        mag = np.where(printed == 0, 1e-300, np.abs(printed))
        tol = np.maximum(0.5001 * 10.0 ** (np.floor(np.log10(mag)) - 5), 1e-12)
        assert np.all(np.abs(got - printed) <= tol)


def test_strain_vs_oracle_random(eng, oracle):
    rng = np.random.default_rng(3)
    from digitalvolumecorrelation_gb300 import synth
    pts = synth.grid_points((7, 7, 7), 9.0, (100.0, 90.0, 80.0)) + rng.normal(0, 0.5, (343, 3))
    disp = 0.01 * (pts - 90.0) + rng.normal(0, 0.01, (343, 3))
    status = np.where(rng.uniform(size=343) < 0.1, -1, 0).astype(np.int32)
    objmin = rng.uniform(0, 0.3, 343)
    _, neigh = oracle.order_neighbours(pts)
    for ndp, objt, refill in ((25, 1.0, False), (40, 0.2, True), (10, 1.0, True)):
        a = eng.strain(pts, status, objmin, disp, neigh, ndp, objt, refill)
        b = oracle.strain(pts, status, objmin, disp, neigh, ndp, objt, refill)
        np.testing.assert_array_equal(a["pts_in_sw"], b["pts_in_sw"])
        # FP64 on both sides, same operations in the same order (the strain
        # kernel is compiled without FMA contraction): bit-identical
        for k in ("u_fit", "sw_radius", "e_strain", "l_strain", "dgrad"):
            np.testing.assert_array_equal(a[k], b[k])


def test_given_seed_mode_vs_oracle(eng, oracle):
    """Independent points with caller seeds (the throughput path) on a larger
    volume, uint8 cube and uint16 sphere."""
    from digitalvolumecorrelation_gb300 import synth
    rng = np.random.default_rng(9)
    shape = (72, 72, 72)
    b = synth.blobs(shape, 500, seed=31)
    aff = synth.Affine(t=(0.8, -1.4, 2.1), E=((0.004, 0.001, 0), (0, -0.003, 0), (0, 0, 0.006)),
                       c=(36.0, 36.0, 36.0))
    ref = synth.render(shape, b, noise_sigma=2.0, noise_seed=32)
    cor = synth.render(shape, b, deform=aff, noise_sigma=2.0, noise_seed=33)
    pts = synth.grid_points((4, 4, 4), 7.0, (36.0, 36.0, 36.0))
    seeds = aff.u(pts) + rng.normal(0, 0.7, pts.shape)
    for kw in (dict(subvol_geom="cube", subvol_size=17, subvol_npts=1000, num_srch_dof=12,
                    disp_max=4, basin_radius=2.0),
               dict(subvol_geom="sphere", subvol_size=19, subvol_npts=1500, num_srch_dof=6,
                    disp_max=4, basin_radius=0.0)):
        from digitalvolumecorrelation_gb300.abi import make_params
        p = make_params(shape, **kw)
        E = eng.Engine(p, ref, cor)
        g = E.process(pts, seed_mode=1, seeds=seeds)
        o = oracle.process(p, ref, cor, pts, seed_mode=1, seeds=seeds)
        np.testing.assert_array_equal(g["status"], o["status"])
        good = o["status"] == 0
        assert np.abs(g["params"][good, :3] - o["params"][good, :3]).max() <= 1e-3
        rel = np.abs(g["objmin"][good] - o["objmin"][good]) / o["objmin"][good]
        assert rel.max() <= 1e-5
        E.close()


def test_two_ctas_per_sm_match_one(eng, monkeypatch):
    """Searches without a coarse grid from independent starts run two CTAs per
    SM at the narrowest cluster width that fits, the correlate region read
    through L1 instead of a staged box: the same search as one CTA per SM
    with staging (12 start parameters given; translation seeds without a
    basin). Widths differ in summation order, and the two compilations of the
    kernel (registers for one or two CTAs) may fuse a multiply and an add
    differently: statuses identical, objmin within 2e-6 relative, parameters
    within 1e-5."""
    from digitalvolumecorrelation_gb300 import synth
    from digitalvolumecorrelation_gb300.abi import make_params
    rng = np.random.default_rng(19)
    shape = (80, 80, 80)  # 80-byte rows: the one-CTA shape stages its region by TMA
    b = synth.blobs(shape, 650, seed=61)
    aff = synth.Affine(t=(0.8, -1.4, 2.1), E=((0.004, 0.001, 0), (0, -0.003, 0), (0, 0, 0.006)),
                       c=(40.0, 40.0, 40.0))
    ref = synth.render(shape, b, noise_sigma=2.0, noise_seed=62)
    cor = synth.render(shape, b, deform=aff, noise_sigma=2.0, noise_seed=63)
    pts = synth.grid_points((4, 4, 4), 7.0, (40.0, 40.0, 40.0))
    p12 = np.zeros((len(pts), 12))
    p12[:, :3] = aff.u(pts) + rng.normal(0, 0.6, pts.shape)
    p12[:, 6:9] = rng.normal(0, 0.003, (len(pts), 3))
    for kw, mode, seeds in ((dict(subvol_geom="cube", subvol_size=19, subvol_npts=2200, num_srch_dof=12,
                                  disp_max=4, basin_radius=2.0), eng.SEED_PARAMS, p12),
                            (dict(subvol_geom="sphere", subvol_size=21, subvol_npts=2500, num_srch_dof=6,
                                  disp_max=4, basin_radius=0.0), eng.SEED_GIVEN, p12[:, :3].copy())):
        E = eng.Engine(make_params(shape, **kw), ref, cor)
        out = {}
        for pair in ("0", "1"):  # one CTA per SM with staging; the default
            if pair == "0":
                monkeypatch.setenv("DVC_PAIR", "0")
            else:
                monkeypatch.delenv("DVC_PAIR", raising=False)
            out[pair] = E.process(pts, seed_mode=mode, seeds=seeds)
            out[pair + "launch"] = E.last_launch()
        assert out["1launch"]["cluster"] == 1  # one CTA holds these subvolumes
        assert out["1launch"]["cluster"] <= out["0launch"]["cluster"]
        assert out["1launch"]["staging"] == 0 and out["0launch"]["staging"] != 0
        assert (out["1"]["status"] == 0).sum() >= 50
        np.testing.assert_array_equal(out["1"]["status"], out["0"]["status"])
        good = out["0"]["status"] == 0
        np.testing.assert_allclose(out["1"]["objmin"][good], out["0"]["objmin"][good], rtol=2e-6, atol=0)
        assert np.abs(out["1"]["params"] - out["0"]["params"]).max() <= 1e-5
        E.close()


def test_subvolume_precheck_vs_oracle(eng, oracle):
    """subvol_thresh as the reference's manual documents it (Core/InputRead.cpp:
    282-323): points whose reference samples lie in the gray range for less
    than min_vol_fract of the samples are not searched (status -3); the rest
    are searched as usual. A dark slab makes some subvolumes fail the check."""
    from digitalvolumecorrelation_gb300 import synth
    from digitalvolumecorrelation_gb300.abi import make_params
    rng = np.random.default_rng(12)
    shape = (72, 72, 72)
    b = synth.blobs(shape, 2500, amp=(60.0, 200.0), seed=51)
    aff = synth.Affine(t=(0.6, -0.9, 1.3), c=(36.0, 36.0, 36.0))
    ref = synth.render(shape, b, noise_sigma=2.0, noise_seed=52)
    cor = synth.render(shape, b, deform=aff, noise_sigma=2.0, noise_seed=53)
    ref[:, :, :30] //= 8  # dark slab, x < 30
    cor[:, :, :31] //= 8
    pts = synth.grid_points((5, 4, 4), 6.0, (36.0, 36.0, 36.0))
    seeds = aff.u(pts) + rng.normal(0, 0.5, pts.shape)
    for geom, size, npts in (("cube", 15, 900), ("sphere", 17, 1200)):
        p = make_params(shape, subvol_geom=geom, subvol_size=size, subvol_npts=npts, num_srch_dof=6,
                        disp_max=3, basin_radius=0.0, subvol_thresh=True, gray_thresh_min=30.0,
                        gray_thresh_max=255.0, min_vol_fract=0.3)
        E = eng.Engine(p, ref, cor)
        g = E.process(pts, seed_mode=1, seeds=seeds)
        o = oracle.process(p, ref, cor, pts, seed_mode=1, seeds=seeds)
        np.testing.assert_array_equal(g["status"], o["status"])
        assert (o["status"] == -3).sum() >= 3 and (o["status"] == 0).sum() >= 10
        good = o["status"] == 0
        assert np.abs(g["params"][good, :3] - o["params"][good, :3]).max() <= 1e-3
        assert np.all(g["params"][~good] == 0.0) and np.all(g["objmin"][~good] == 0.0)
        E.close()


def test_volume_files_streamed_to_the_gpu(eng, tmp_path):
    """dvc_gpu_create_from_files / dvc_gpu_load_raw: raw files with a header
    and big-endian 16-bit data give the same volume (and so the same search)
    as the host-buffer upload; larger than one 64 MiB staging chunk."""
    import torch
    from digitalvolumecorrelation_gb300 import synth
    from digitalvolumecorrelation_gb300.abi import make_params
    shape = (512, 256, 300)  # 75 MiB of uint16
    rng = np.random.default_rng(3)
    vol = rng.integers(0, 65535, size=shape[::-1], dtype=np.uint16)
    hdr = b"\x07" * 37
    path = tmp_path / "vol.raw"
    path.write_bytes(hdr + vol.astype(">u2").tobytes())
    dev = torch.zeros(vol.size + 32, dtype=torch.int16, device="cuda")
    eng.load_raw(dev, str(path), shape, 2, header_bytes=len(hdr), big_endian=True)
    got = dev[: vol.size].cpu().numpy().view(np.uint16).reshape(vol.shape)
    np.testing.assert_array_equal(got, vol)
    # a small pair through the engine: same results as the host upload
    small = (48, 48, 48)
    b = synth.blobs(small, 250, seed=61)
    ref = synth.render(small, b, noise_seed=62, dtype=np.uint16, vmax=65535)
    cor = synth.render(small, b, deform=synth.Affine(t=(0.7, -0.4, 1.1)), noise_seed=63, dtype=np.uint16,
                       vmax=65535)
    (tmp_path / "r.raw").write_bytes(hdr + ref.astype(">u2").tobytes())
    (tmp_path / "c.raw").write_bytes(hdr + cor.astype(">u2").tobytes())
    p = make_params(small, bytes_per_voxel=2, subvol_size=13, subvol_npts=500, disp_max=3)
    pts = synth.grid_points((3, 3, 3), 6.0, (24.0, 24.0, 24.0))
    seeds = np.tile([0.7, -0.4, 1.1], (len(pts), 1))
    E1 = eng.Engine(p, ref.astype(">u2").view(np.uint16), cor.astype(">u2").view(np.uint16), big_endian=True)
    E2 = eng.Engine(p, ref_path=str(tmp_path / "r.raw"), cor_path=str(tmp_path / "c.raw"),
                    header_bytes=len(hdr), big_endian=True)
    r1 = E1.process(pts, seed_mode=1, seeds=seeds)
    r2 = E2.process(pts, seed_mode=1, seeds=seeds)
    for k in ("status", "objmin", "params"):
        np.testing.assert_array_equal(r1[k], r2[k])
    assert (r1["status"] == 0).all()
    E1.close()
    E2.close()


@pytest.mark.parametrize("bpv,step,cluster", [(1, 3, None), (2, 4, None), (2, 3, 8)])
def test_whole_voxel_grid_vs_oracle(eng, oracle, bpv, step, cluster):
    """The 5 x 5 x 5 grid with a whole-voxel step of 3 or 4 against the
    oracle, from seeds up to two steps off the truth, uint8 and uint16, cube
    and sphere. One CTA per point evaluates it by thread groups of one chunk
    with shared sample records; clusters of 8 leave at most ~190 samples per
    CTA, too few for the record area, so the 32-lane groups with shuffles
    evaluate it."""
    from digitalvolumecorrelation_gb300 import synth
    from digitalvolumecorrelation_gb300.abi import make_params
    rng = np.random.default_rng(70 + step)
    shape = (96, 96, 96)
    b = synth.blobs(shape, 3000, amp=(60.0, 200.0), seed=71)
    aff = synth.Affine(t=(1.2, -0.7, 0.4), E=((0.004, 0.0, 0.0), (0.0, -0.003, 0.0), (0.0, 0.0, 0.005)),
                       c=(48.0, 48.0, 48.0))
    dt = np.uint8 if bpv == 1 else np.uint16
    vmax = 255 if bpv == 1 else 65535
    ref = synth.render(shape, b, noise_sigma=2.0, noise_seed=72, dtype=dt, vmax=vmax)
    cor = synth.render(shape, b, deform=aff, noise_sigma=2.0, noise_seed=73, dtype=dt, vmax=vmax)
    pts = synth.grid_points((4, 4, 3), 7.0, (48.0, 48.0, 48.0))
    seeds = aff.u(pts) + rng.integers(-2, 3, pts.shape) * step + rng.normal(0, 0.3, pts.shape)
    for geom, size, npts in (("cube", 15, 1000), ("sphere", 17, 1400)):
        p = make_params(shape, bytes_per_voxel=bpv, subvol_geom=geom, subvol_size=size, subvol_npts=npts,
                        num_srch_dof=6, disp_max=2 * step, basin_radius=float(step))
        E = eng.Engine(p, ref, cor)
        if cluster:
            E.set_cluster(cluster)
        g = E.process(pts, seed_mode=1, seeds=seeds)
        E.close()
        o = oracle.process(p, ref, cor, pts, seed_mode=1, seeds=seeds)
        for r in (g,):
            np.testing.assert_array_equal(r["status"], o["status"])
            good = o["status"] == 0
            assert good.mean() > 0.8
            assert np.abs(r["params"][good, :3] - o["params"][good, :3]).max() <= 1e-3
            rel = np.abs(r["objmin"][good] - o["objmin"][good]) / np.abs(o["objmin"][good])
            assert rel.max() <= 1e-5


def test_grid_with_slab_staging_vs_oracle(eng, oracle):
    """Cube 41 / 3375 samples, uint16, 5 x 5 x 5 grid of step 3, at cluster
    width 4: the box covering every translation does not fit beside the
    sample state, so the grid stages one z slab of translations at a time.
    Against the oracle, from seeds up to two steps off the truth."""
    from digitalvolumecorrelation_gb300 import synth
    from digitalvolumecorrelation_gb300.abi import make_params
    rng = np.random.default_rng(81)
    shape = (112, 112, 112)
    b = synth.blobs(shape, 4000, amp=(2000.0, 60000.0), seed=82)
    aff = synth.Affine(t=(0.9, -1.3, 0.6), E=((0.003, 0.0, 0.0), (0.0, 0.002, 0.0), (0.0, 0.0, -0.004)),
                       c=(56.0, 56.0, 56.0))
    ref = synth.render(shape, b, noise_sigma=150.0, noise_seed=83, dtype=np.uint16, vmax=65535)
    cor = synth.render(shape, b, deform=aff, noise_sigma=150.0, noise_seed=84, dtype=np.uint16, vmax=65535)
    pts = synth.grid_points((2, 2, 2), 10.0, (56.0, 56.0, 56.0))
    seeds = aff.u(pts) + rng.integers(-2, 3, pts.shape) * 3 + rng.normal(0, 0.3, pts.shape)
    p = make_params(shape, bytes_per_voxel=2, subvol_geom="cube", subvol_size=41, subvol_npts=3000,
                    num_srch_dof=6, disp_max=6, basin_radius=3.0)
    E = eng.Engine(p, ref, cor)
    E.set_cluster(4)
    g = E.process(pts, seed_mode=1, seeds=seeds)
    launch = E.last_launch()
    E.close()
    assert launch["cluster"] == 4 and launch["staging"] == 2
    o = oracle.process(p, ref, cor, pts, seed_mode=1, seeds=seeds)
    np.testing.assert_array_equal(g["status"], o["status"])
    good = o["status"] == 0
    assert good.all()
    assert np.abs(g["params"][good, :3] - o["params"][good, :3]).max() <= 1e-3
    rel = np.abs(g["objmin"][good] - o["objmin"][good]) / np.abs(o["objmin"][good])
    assert rel.max() <= 1e-5


def test_wide_grid_without_slab_staging_vs_oracle(eng, oracle):
    """A 13 x 13 x 13 grid (disp_max 6, basin_radius 1) on cube 41 / 3375
    samples, uint16, asked for cluster width 4: its box does not fit there,
    and a z slab of 169 translations is more than one grid chunk, so the
    engine widens the cluster (or leaves the region unstaged) instead of
    staging slabs. Against the oracle, from seeds up to four voxels off the
    truth."""
    from digitalvolumecorrelation_gb300 import synth
    from digitalvolumecorrelation_gb300.abi import make_params
    rng = np.random.default_rng(91)
    shape = (112, 112, 112)
    b = synth.blobs(shape, 4000, amp=(2000.0, 60000.0), seed=92)
    aff = synth.Affine(t=(-0.8, 1.1, 0.5), E=((0.002, 0.0, 0.0), (0.0, -0.003, 0.0), (0.0, 0.0, 0.002)),
                       c=(56.0, 56.0, 56.0))
    ref = synth.render(shape, b, noise_sigma=150.0, noise_seed=93, dtype=np.uint16, vmax=65535)
    cor = synth.render(shape, b, deform=aff, noise_sigma=150.0, noise_seed=94, dtype=np.uint16, vmax=65535)
    pts = synth.grid_points((2, 2, 1), 10.0, (56.0, 56.0, 56.0))
    seeds = aff.u(pts) + rng.integers(-4, 5, pts.shape) + rng.normal(0, 0.3, pts.shape)
    p = make_params(shape, bytes_per_voxel=2, subvol_geom="cube", subvol_size=41, subvol_npts=3000,
                    num_srch_dof=6, disp_max=6, basin_radius=1.0)
    E = eng.Engine(p, ref, cor)
    E.set_cluster(4)
    g = E.process(pts, seed_mode=1, seeds=seeds)
    launch = E.last_launch()
    E.close()
    assert launch["staging"] != 2
    o = oracle.process(p, ref, cor, pts, seed_mode=1, seeds=seeds)
    np.testing.assert_array_equal(g["status"], o["status"])
    good = o["status"] == 0
    assert good.all()
    assert np.abs(g["params"][good, :3] - o["params"][good, :3]).max() <= 1e-3
    rel = np.abs(g["objmin"][good] - o["objmin"][good]) / np.abs(o["objmin"][good])
    assert rel.max() <= 1e-5

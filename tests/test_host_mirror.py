"""Host logic of the reference-API mirror (no GPU): rounding, source scaling,
the L2 misfit and the checks the reference asserts."""
import numpy as np
import pytest


def test_nearest_grid_points_ties_up(sw):
    # RoundNearestTiesUp of pos/h + 1
    idx = sw.nearest_grid_points(np.array([[2.5, 7.5], [0.0, 12.49], [4.999, 5.0]]), (5.0, 5.0))
    assert idx.tolist() == [[2, 3], [1, 3], [2, 2]]
    assert idx.dtype == np.int32 and idx.flags.f_contiguous


def test_scale_srctf(sw):
    vp = np.asfortranarray(np.arange(1, 13, dtype=float).reshape(3, 4, order="F") * 100)
    tf = np.ones((5, 2))
    si = np.array([[2, 3], [1, 1]], dtype=np.int32)
    out = sw.scale_srctf(tf, si, vp, (2.0, 4.0), 1e-3)
    assert out.dtype == np.float32
    np.testing.assert_allclose(out[:, 0], 1e-6 / 8.0 * vp[1, 2] ** 2, rtol=1e-6)
    np.testing.assert_allclose(out[:, 1], 1e-6 / 8.0 * vp[0, 0] ** 2, rtol=1e-6)


def test_l2_misfit(sw):
    rng = np.random.default_rng(0)
    obs = rng.standard_normal((50, 3))
    syn = rng.standard_normal((50, 3))
    recs = sw.ScalarReceivers(np.zeros((3, 2)), 50)
    recs.seismograms[...] = syn
    ic = rng.uniform(0.5, 2, 50)
    m = sw.L2Misfit(observed=obs, invcov=np.diag(ic), windows=[(5, 20), (30, 40)])
    mask = np.zeros(50)
    mask[4:20] = 1
    mask[29:40] = 1
    r = mask[:, None] * (syn - obs)
    assert np.isclose(m.calcmisfit(recs), 0.5 * np.sum(r * ic[:, None] * r))
    np.testing.assert_allclose(m.dchi_du(recs), ic[:, None] * r)
    np.testing.assert_allclose(m.invcov_diagonal(), ic)
    assert m.invcov_dense() is None
    dense = sw.L2Misfit(observed=obs, invcov=np.ones((50, 50)))
    assert dense.invcov_diagonal() is None
    assert dense.invcov_dense().shape == (50, 50)
    with pytest.raises(AssertionError):
        sw.L2Misfit(observed=obs, windows=[(0, 3)])


def test_parameter_checks(sw):
    with pytest.raises(AssertionError, match="positive"):
        sw.InputParametersAcoustic(0, 1e-3, (10, 10), (1.0, 1.0), sw.CPMLBoundaryConditionParameters())
    with pytest.raises(AssertionError):
        sw.GradParameters(check_freq=0)
    with pytest.raises(AssertionError, match="at least one source"):
        sw.ScalarSources(np.zeros((0, 2)), np.zeros((10, 0)), 5.0)
    assert sw.courant_number(np.full((3, 3), 2000.0), 1e-3, (5.0, 5.0)) == pytest.approx(2000 * 1e-3 * np.sqrt(0.08))
    assert sw.points_per_wavelength(np.full((3, 3), 1500.0), (10.0, 8.0), 8.0) == pytest.approx(1500 / 160)


def test_vd_source_scaling_and_cfl(sw):
    """possrcrec_scaletf of the VD simulation (tf * dt * vp^2 rho / prod(h),
    acou_forward.jl:66-80) and its CFL number with the 7/6 factor (acou_models.jl:240-251)."""
    import importlib
    V = importlib.import_module(sw.__name__ + ".vd")
    vp = np.asfortranarray(np.arange(1, 13, dtype=float).reshape(3, 4, order="F") * 100)
    rho = np.asfortranarray(1000.0 + np.arange(12, dtype=float).reshape(3, 4, order="F"))
    tf = np.ones((5, 2))
    si = np.array([[2, 3], [1, 1]], dtype=np.int32)
    out = V.scale_srctf_vd(tf, si, vp, rho, (2.0, 4.0), 1e-3)
    assert out.dtype == np.float32
    np.testing.assert_allclose(out[:, 0], 1e-3 / 8.0 * vp[1, 2] ** 2 * rho[1, 2], rtol=1e-6)
    np.testing.assert_allclose(out[:, 1], 1e-3 / 8.0 * vp[0, 0] ** 2 * rho[0, 0], rtol=1e-6)
    c = V.vd_courant_number(vp, 1e-3, (2.0, 4.0))
    assert c == pytest.approx(1200.0 * 1e-3 * np.sqrt(1 / 4 + 1 / 16) * 7 / 6)
    mp = sw.VpRhoAcousticVDMaterialProperties(vp, rho)
    assert mp.interp_method.code == 0
    assert sw.VpRhoAcousticVDMaterialProperties(vp, rho, sw.HarmonicAverageInterpolation()).interp_method.code == 1


def test_vd_and_ccts_shot_consistency(sw):
    """check_sim_consistency accepts scalar shots for VD material properties
    and rejects vector receivers; CCTSMisfit keeps the reference's arguments."""
    from seismicwaves_gb300 import api
    vp = np.full((10, 8), 2000.0)
    mp = sw.VpRhoAcousticVDMaterialProperties(vp, np.full((10, 8), 1800.0))
    shot = sw.ScalarShot(srcs=sw.ScalarSources(np.array([[20.0, 20.0]]), np.ones((10, 1)), 10.0),
                         recs=sw.ScalarReceivers(np.array([[30.0, 10.0]]), 10))
    api._check_sim_consistency(mp, [shot])
    bad = sw.ScalarShot(srcs=shot.srcs, recs=sw.VectorReceivers(np.array([[30.0, 10.0]]), 10))
    with pytest.raises(TypeError):
        api._check_sim_consistency(mp, [bad])
    m = sw.CCTSMisfit(1e-3, std=2.0, observed=np.zeros((10, 1)))
    assert m.kind == 1 and m.dt == 1e-3 and m.std == 2.0
    assert m.invcov_diagonal() is None and m.invcov_dense() is None and m.windows == []
    with pytest.raises(AssertionError):
        sw.CCTSMisfit(0.0, observed=np.zeros((10, 1)))


def test_elastic_host_checks(sw):
    """The elastic mirror keeps the reference's argument checks
    (src/models/elastic/ela_params.jl:27-31, src/shots/sources.jl:71-86,
    src/shots/receivers.jl:89) and material defaults
    (ela_material_properties.jl:9-22: arithmetic rho and mu, harmonic lambda)."""
    E = __import__(sw.__name__ + ".elastic", fromlist=["elastic"])
    bc = sw.CPMLBoundaryConditionParameters()
    with pytest.raises(AssertionError, match="Dimensionality"):
        E.InputParametersElastic(10, 1e-3, (4, 4, 4, 4), (1.0,) * 4, bc)
    with pytest.raises(AssertionError, match="grid points must be positive"):
        E.InputParametersElastic(10, 1e-3, (4, 0), (1.0, 1.0), bc)
    with pytest.raises(AssertionError, match="grid spacings must be positive"):
        E.InputParametersElastic(10, 1e-3, (4, 4), (1.0, 0.0), bc)
    with pytest.raises(AssertionError, match="timesteps must be positive"):
        E.InputParametersElastic(0, 1e-3, (4, 4), (1.0, 1.0), bc)
    with pytest.raises(AssertionError, match="Timestep size must be positive"):
        E.InputParametersElastic(10, 0.0, (4, 4), (1.0, 1.0), bc)
    pos = np.array([[10.0, 10.0], [20.0, 10.0]])
    with pytest.raises(AssertionError, match="at least one source"):
        E.MomentTensorSources(np.zeros((0, 2)), np.zeros((5, 0)), [], 10.0)
    with pytest.raises(AssertionError, match="do not match between positions and time-functions"):
        E.MomentTensorSources(pos, np.zeros((5, 3)), [E.MomentTensor2D(1, 1, 0)] * 2, 10.0)
    with pytest.raises(AssertionError, match="moment tensors must match"):
        E.MomentTensorSources(pos, np.zeros((5, 2)), [E.MomentTensor2D(1, 1, 0)], 10.0)
    with pytest.raises(AssertionError, match="components do not match"):
        E.ExternalForceSources(pos, np.zeros((5, 3, 2)), 10.0)
    with pytest.raises(AssertionError, match="at least one receiver"):
        E.VectorReceivers(np.zeros((0, 2)), 5)
    assert E.VectorReceivers(pos, 7).seismograms.shape == (7, 2, 2)
    m = E.ElasticIsoMaterialProperties(np.ones((3, 3)), np.ones((3, 3)), np.ones((3, 3)))
    assert (m.interp_method_ρ.code, m.interp_method_λ.code, m.interp_method_μ.code) == (0, 1, 0)


def test_elastic_shot_consistency_and_build_routing(sw):
    """check_sim_consistency (src/utils/checks.jl:2-41) for elastic shots, and
    build_wavesim's argument errors, which come before any device work."""
    from seismicwaves_gb300 import api
    E = __import__(sw.__name__ + ".elastic", fromlist=["elastic"])
    m = E.ElasticIsoMaterialProperties(np.ones((8, 8)), np.ones((8, 8)), np.ones((8, 8)))
    pos = np.array([[10.0, 10.0]])
    mt = E.MomentTensorShot(srcs=E.MomentTensorSources(pos, np.zeros((5, 1)), [E.MomentTensor2D(1, 1, 0)], 10.0),
                            recs=E.VectorReceivers(pos, 5))
    ef = E.ExternalForceShot(srcs=E.ExternalForceSources(pos, np.zeros((5, 2, 1)), 10.0),
                             recs=E.VectorReceivers(pos, 5))
    api._check_sim_consistency(m, [mt, mt])
    api._check_sim_consistency(m, [ef])
    with pytest.raises(TypeError):
        api._check_sim_consistency(m, [mt, ef])
    scalar = E.MomentTensorShot(srcs=mt.srcs, recs=sw.ScalarReceivers(pos, 5))
    with pytest.raises(TypeError):
        api._check_sim_consistency(m, [scalar])
    params = sw.InputParametersAcoustic(10, 1e-3, (8, 8), (1.0, 1.0), sw.CPMLBoundaryConditionParameters())
    vp = sw.VpAcousticCDMaterialProperties(np.full((8, 8), 2000.0))
    with pytest.raises(ValueError, match="threadpersrc"):
        sw.build_wavesim(params, vp, runparams=sw.RunParameters(parall="threadpersrc"))
    with pytest.raises(AssertionError, match="gradient keyword"):
        sw.build_wavesim(params, vp, runparams=sw.RunParameters(), gradparams=sw.GradParameters(), gradient=False)

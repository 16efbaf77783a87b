"""Known-answer tests of the oracle's shading restatement (oracle/shading.h,
oracle/pathtracer.cpp): Fresnel at normal incidence and total internal
reflection, the Lambert estimator and white furnace, pdf normalisation and
sample/evaluation consistency of the GGX conductor and rough dielectric
(legacy stretched visible-normal sampling, microfacet.h:86-164), conductor
reciprocity, the Henyey-Greenstein phase function (media.cpp:83-111),
area-light sampling against a triangle's solid angle, and a closed emissive
Lambertian sphere whose radiance is Le / (1 - albedo).

These pin the restatement to analytic answers; the reference itself cannot be
built here, so they are the oracle's anchor for T9-T13 and T17."""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = []


def _sphere_grid(n_theta: int, n_phi: int):
    """Midpoint grid over the unit sphere: directions [n, 3] and solid angles [n]."""
    th = (np.arange(n_theta) + 0.5) * np.pi / n_theta
    ph = (np.arange(n_phi) + 0.5) * 2 * np.pi / n_phi
    T, P = np.meshgrid(th, ph, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
    dw = (np.sin(T) * (np.pi / n_theta) * (2 * np.pi / n_phi)).reshape(-1)
    return d.astype(np.float32), dw


def _dir(theta_deg: float, phi_deg: float = 30.0) -> np.ndarray:
    t, p = np.radians(theta_deg), np.radians(phi_deg)
    return np.array([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)], np.float32)


# ------------------------------------------------------------------ Fresnel
@pytest.mark.parametrize("eta", [1.33, 1.5, 2.4])
def test_fresnel_dielectric_normal_incidence_and_total_reflection(oracle_lib, eta):
    assert O.fr_dielectric(1.0, eta) == pytest.approx(((eta - 1) / (eta + 1)) ** 2, rel=1e-5)
    assert O.fr_dielectric(-1.0, eta) == pytest.approx(((eta - 1) / (eta + 1)) ** 2, rel=1e-5)
    # from inside beyond the critical angle: everything is reflected
    crit = np.sqrt(1 - 1 / eta ** 2)   # cos of the critical angle
    assert O.fr_dielectric(-0.5 * crit, eta) == 1.0
    # the same interface seen from the refracted side reflects the same fraction
    for cos_i in (0.9, 0.6, 0.3):
        sin_t = np.sqrt(1 - cos_i ** 2) / eta
        cos_t = np.sqrt(1 - sin_t ** 2)
        assert O.fr_dielectric(cos_i, eta) == pytest.approx(O.fr_dielectric(-cos_t, eta), rel=1e-4)


def test_conductor_fresnel_at_normal_incidence(oracle_lib):
    """A smooth conductor reflects F = ((eta-1)^2 + k^2) / ((eta+1)^2 + k^2) at
    normal incidence, k = 2 sqrt(r) / sqrt(1 - r) from its colour r
    (conductor.h:12-93)."""
    color = np.array([0.9, 0.5, 0.2], np.float32)
    eta = 1.5
    m = O.material(O.MAT_CONDUCTOR, color, roughness=0.0, ior=eta)
    s = O.bsdf_sample(m, _dir(0.0), np.zeros((1, 3), np.float32))[0]
    k = 2 * np.sqrt(color) / np.sqrt(1 - color)
    want = ((eta - 1) ** 2 + k ** 2) / ((eta + 1) ** 2 + k ** 2)
    np.testing.assert_allclose(s[0:3] * abs(s[5]), want, rtol=1e-4)
    assert s[6] == 1.0 and np.allclose(s[3:6], [0, 0, 1], atol=1e-6)


# ------------------------------------------------------------------ Lambert
def test_lambert_estimator_is_the_albedo_and_pdf_is_normalised(oracle_lib):
    albedo = (0.63, 0.065, 0.05)
    m = O.material(O.MAT_DIFFUSE, albedo)
    u = np.random.default_rng(1).random((4096, 3), dtype=np.float32)
    for wo in (_dir(10.0), _dir(70.0), -_dir(40.0)):
        s = O.bsdf_sample(m, wo, u)
        ok = s[:, 6] > 0
        assert ok.mean() > 0.999
        est = s[ok, 0:3] * np.abs(s[ok, 5:6]) / s[ok, 6:7]
        np.testing.assert_allclose(est, np.broadcast_to(albedo, est.shape), rtol=2e-5)
        assert np.all(np.sign(s[ok, 5]) == np.sign(wo[2]))
    d, dw = _sphere_grid(400, 800)
    pdf = O.bsdf_eval(m, _dir(25.0), d)[:, 3]
    assert float(np.sum(pdf * dw)) == pytest.approx(1.0, abs=2e-4)


# --------------------------------------------------------- GGX conductor
@pytest.mark.parametrize("roughness", [0.5, 0.8, 1.0])
@pytest.mark.parametrize("theta", [5.0, 45.0, 75.0])
def test_ggx_conductor_pdf_sampling_and_energy(oracle_lib, roughness, theta):
    """The pdf integrates over the sphere to the fraction of samples that
    stay above the surface; a sample's f and pdf equal the evaluated ones;
    a white conductor (r -> 1, F -> 1) never reflects more than it receives."""
    wo = _dir(theta)
    m = O.material(O.MAT_CONDUCTOR, (0.9999, 0.9999, 0.9999), roughness=roughness, ior=1.5)
    d, dw = _sphere_grid(1200, 2400)
    ev = O.bsdf_eval(m, wo, d)
    integral = float(np.sum(ev[:, 3] * dw))
    u = np.random.default_rng(int(theta * 10 + roughness * 100)).random((200000, 3), dtype=np.float32)
    s = O.bsdf_sample(m, wo, u)
    valid = s[:, 6] > 0
    frac = float(valid.mean())
    assert integral <= 1.0 + 2e-3
    assert integral == pytest.approx(frac, abs=4e-3 + 4 * np.sqrt(frac * (1 - frac) / u.shape[0]))
    # sample / evaluation consistency
    re = O.bsdf_eval(m, wo, s[valid, 3:6])
    np.testing.assert_allclose(re[:, 3], s[valid, 6], rtol=2e-3, atol=1e-6)
    np.testing.assert_allclose(re[:, 0:3], s[valid, 0:3], rtol=2e-3, atol=1e-6)
    # white furnace: the sampled estimate E[f cos / pdf] equals the directional
    # albedo integrated on the grid, and stays below 1 (single scattering loses
    # the energy of reflections below the horizon, most at high roughness)
    albedo = float(np.sum(s[valid, 0] * np.abs(s[valid, 5]) / s[valid, 6]) / u.shape[0])
    grid_albedo = float(np.sum(ev[:, 0] * np.abs(d[:, 2]) * dw))
    assert albedo == pytest.approx(grid_albedo, abs=5e-3)
    assert grid_albedo <= 1.0 + 2e-3
    if roughness <= 0.5:
        assert grid_albedo > 0.83


def test_ggx_at_unit_roughness_loses_half_its_samples_at_normal_incidence(oracle_lib):
    """With alpha = 1 the GGX distribution is uniform (D = 1/pi), so at
    normal incidence the visible normals are cosine-distributed and a
    reflection stays above the surface exactly when the normal is within
    45 degrees of the axis: probability sin^2(45 deg) = 1/2."""
    m = O.material(O.MAT_CONDUCTOR, (0.9999, 0.9999, 0.9999), roughness=1.0, ior=1.5)
    wo = np.array([0.0, 0.0, 1.0], np.float32)
    d, dw = _sphere_grid(1500, 3000)
    assert float(np.sum(O.bsdf_eval(m, wo, d)[:, 3] * dw)) == pytest.approx(0.5, abs=2e-3)
    u = np.random.default_rng(9).random((400000, 3), dtype=np.float32)
    assert float((O.bsdf_sample(m, wo, u)[:, 6] > 0).mean()) == pytest.approx(0.5, abs=4e-3)


def test_ggx_conductor_is_reciprocal(oracle_lib):
    rng = np.random.default_rng(7)
    m = O.material(O.MAT_CONDUCTOR, (0.9, 0.6, 0.3), roughness=0.6, ior=1.3)
    wo = rng.normal(size=(2000, 3)).astype(np.float32)
    wi = rng.normal(size=(2000, 3)).astype(np.float32)
    wo[:, 2], wi[:, 2] = np.abs(wo[:, 2]) + 0.05, np.abs(wi[:, 2]) + 0.05
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    a = O.bsdf_eval(m, wo, wi)[:, 0:3]
    b = O.bsdf_eval(m, wi, wo)[:, 0:3]
    assert np.all(a > 0)
    np.testing.assert_allclose(a, b, rtol=1e-4)


# ---------------------------------------------------- rough dielectric
@pytest.mark.parametrize("roughness", [0.5, 0.9])
@pytest.mark.parametrize("wo", [_dir(20.0), -_dir(50.0)])
def test_rough_dielectric_pdf_and_sampling(oracle_lib, roughness, wo):
    """A sample carries the evaluated f; its pdf is the evaluated one with the
    reflect/refract choice made on F at the sampled microfacet normal, where
    the reference's pdf() takes F at the shading normal (dielectric.h:166
    against :229; the restatement keeps both); the reflection part is
    reciprocal; the evaluated pdf integrates to at most 1."""
    eta = 1.5
    m = O.material(O.MAT_DIELECTRIC, (1.0, 1.0, 1.0), roughness=roughness, spec_trans=1.0, ior=eta)
    d, dw = _sphere_grid(1200, 2400)
    assert float(np.sum(O.bsdf_eval(m, wo, d)[:, 3] * dw)) <= 1.0 + 3e-3
    u = np.random.default_rng(3).random((50000, 3), dtype=np.float32)
    s = O.bsdf_sample(m, wo, u)
    valid = s[:, 6] > 0
    assert valid.mean() > 0.7
    sv = s[valid]
    re = O.bsdf_eval(m, wo, sv[:, 3:6])
    np.testing.assert_allclose(re[:, 0:3], sv[:, 0:3], rtol=3e-3, atol=1e-6)
    refl = np.sign(sv[:, 5]) == np.sign(wo[2])
    assert refl.any() and (~refl).any()
    # microfacet normal of each sample (generalised half vector)
    etap = np.where(refl, 1.0, eta if wo[2] > 0 else 1 / eta)
    wm = sv[:, 3:6] * etap[:, None] + wo
    wm /= np.linalg.norm(wm, axis=1, keepdims=True)
    wm *= np.sign(wm[:, 2:3])
    f_m = np.array([O.fr_dielectric(float(np.copysign(np.dot(wo, x), wo[2])), eta) for x in wm])
    f_n = O.fr_dielectric(float(wo[2]), eta)
    sel_sample = np.where(refl, f_m, 1 - f_m)
    sel_eval = np.where(refl, f_n, 1 - f_n)
    np.testing.assert_allclose(sv[:, 6] * sel_eval, re[:, 3] * sel_sample, rtol=3e-3, atol=1e-7)
    back = O.bsdf_eval(m, sv[refl, 3:6], np.broadcast_to(wo, (int(refl.sum()), 3)))[:, 0:3]
    np.testing.assert_allclose(back, sv[refl, 0:3], rtol=3e-3, atol=1e-6)


def test_smooth_dielectric_splits_by_fresnel(oracle_lib):
    """A smooth dielectric reflects with probability F and refracts by Snell's law."""
    eta = 1.5
    m = O.material(O.MAT_DIELECTRIC, (1.0, 1.0, 1.0), roughness=0.0, spec_trans=1.0, ior=eta)
    wo = _dir(40.0)
    F = O.fr_dielectric(float(wo[2]), eta)
    u = np.random.default_rng(5).random((100000, 3), dtype=np.float32)
    s = O.bsdf_sample(m, wo, u)
    refl = s[:, 5] > 0
    assert refl.mean() == pytest.approx(F, abs=4 * np.sqrt(F * (1 - F) / u.shape[0]))
    t = s[~refl][0]
    sin_i = np.sqrt(1 - wo[2] ** 2)
    assert np.sqrt(1 - t[5] ** 2) == pytest.approx(sin_i / eta, rel=1e-5)


# ------------------------------------------------------------------ HG
@pytest.mark.parametrize("g", [-0.5, 0.0, 0.3, 0.8])
def test_henyey_greenstein_normalised_mean_cosine_and_sampling(oracle_lib, g):
    wo = _dir(30.0)
    d, dw = _sphere_grid(1000, 2000)
    p = np.array([O.hg_p(g, wo, x) for x in d[:: 97]])
    # the full grid through the sampled path: every pdf value against hg_p
    u = np.random.default_rng(11).random((200000, 2), dtype=np.float32)
    s = O.hg_sample(g, wo, u)
    for k in range(0, 200000, 20011):
        assert s[k, 3] == pytest.approx(O.hg_p(g, wo, s[k, 0:3]), rel=1e-5)
    # normalisation, by the closed form on the grid
    cosang = d @ wo
    gg = np.clip(g, -0.99, 0.99)
    pf = (1 - gg * gg) / (4 * np.pi * (1 + gg * gg + 2 * gg * cosang) ** 1.5)
    np.testing.assert_allclose(p, pf[:: 97], rtol=1e-4)
    assert float(np.sum(pf * dw)) == pytest.approx(1.0, abs=1e-3)
    # the restatement samples -wo's lobe: the mean cosine with wo is -g
    # (wo points away from the scattering point, as in the reference)
    mean_cos = float(np.mean(s[:, 0:3] @ wo))
    assert mean_cos == pytest.approx(-g, abs=5e-3)


# ------------------------------------------------------------ area lights
def _solid_angle(a, b, c):
    """Solid angle of a triangle seen from the origin (Van Oosterom and Strackee 1983)."""
    la, lb, lc = (np.linalg.norm(v) for v in (a, b, c))
    num = abs(np.dot(a, np.cross(b, c)))
    den = la * lb * lc + np.dot(a, b) * lc + np.dot(a, c) * lb + np.dot(b, c) * la
    return 2 * np.arctan2(num, den)


def test_area_light_sampling_solid_angle_and_one_sided_emission(oracle_lib):
    """Uniform area sampling of an emissive triangle under an instance
    transform (shape.h:54-123, light.h:167-193): E[1 / pdf] over samples is
    the triangle's solid angle, the sampled pdf equals the one the hit side
    uses for MIS, samples lie on the triangle, and the triangle emits only
    towards the side its normal faces."""
    from kiraray_gb300 import _lib as L
    from kiraray_gb300 import scenes

    pos = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]], np.float32)  # normal +z
    nrm = np.tile(np.array([0.0, 0.0, 1.0], np.float32), (3, 1))
    le = (5.0, 4.0, 3.0)
    mesh = scenes.Mesh(pos, nrm, np.array([[0, 1, 2]], np.uint32), material=0, emission=le)
    xf = scenes._xform((2.0, 1.5, 1.0), 30.0, (0.3, -0.2, 0.5))
    cam = scenes._camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 40.0, 8, 8)
    sc = scenes.Scene([mesh], [(0, xf)], [scenes.Material(type=L.MATERIAL_DIFFUSE)], cam, 8, 8)
    pt = O.PathTracer(sc)
    assert pt.light_count() == 1
    world = (xf[:, :3].astype(np.float64) @ pos.T.astype(np.float64)).T + xf[:, 3]
    n_world = np.cross(world[1] - world[0], world[2] - world[0])
    n_world /= np.linalg.norm(n_world)
    centre = world.mean(0)
    u = np.random.default_rng(21).random((200000, 2), dtype=np.float32)
    for side, cp in ((1, centre + 1.3 * n_world + np.array([0.2, 0.1, -0.3])),
                     (-1, centre - 0.9 * n_world + np.array([-0.1, 0.3, 0.2]))):
        s = pt.light_sample(0, cp.astype(np.float32), u)
        assert np.all(s[:, 6] > 0)
        np.testing.assert_allclose(s[:, 7], s[:, 6], rtol=1e-4)
        est = 1.0 / s[:, 6].astype(np.float64)
        omega = _solid_angle(*(world - cp))
        assert est.mean() == pytest.approx(omega, abs=4 * est.std() / np.sqrt(est.size))
        # on the triangle: in its plane, barycentrics in [0, 1]
        p = s[:, 0:3].astype(np.float64)
        assert np.abs((p - world[0]) @ n_world).max() < 1e-5
        e1, e2, q = world[1] - world[0], world[2] - world[0], p - world[0]
        g = np.array([[e1 @ e1, e1 @ e2], [e1 @ e2, e2 @ e2]])
        b = np.linalg.solve(g, np.stack([q @ e1, q @ e2]))
        assert b.min() > -1e-5 and (b.sum(0)).max() < 1 + 1e-5
        want = np.array(le) if side > 0 else np.zeros(3)
        np.testing.assert_allclose(s[:, 3:6], np.broadcast_to(want, (u.shape[0], 3)), rtol=1e-6)


# ------------------------------------------------- closed-sphere furnace
@pytest.mark.parametrize("nee", [1, 0])
def test_closed_lambertian_sphere_radiance(oracle_lib, nee):
    """Inside a closed sphere whose surface emits Le and reflects with
    Lambertian albedo a, the radiance is Le / (1 - a) everywhere (here up to
    max_depth bounces: Le (1 - a^(D+1)) / (1 - a))."""
    from tests.helpers import furnace_sphere

    sc, want = furnace_sphere()
    pt = O.PathTracer(sc)
    acc = np.zeros(3)
    frames = 48
    for f in range(1, frames + 1):
        Lrad, _ = pt.render({"max_depth": sc.max_depth, "nee": nee, "spp": 1}, f)
        acc += Lrad.mean(axis=0)
    np.testing.assert_allclose(acc / frames, want, rtol=0.02)

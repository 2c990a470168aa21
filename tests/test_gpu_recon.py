"""Device reconstruction from moments: Kubo-Bastin sigma(Ef) and the DOS,
against the oracle's restatements of src/applications/conductivity.jl:101-157
and src/applications/dos.jl:76-161, plus the quantised Haldane Hall
conductance of test/kubo_bastin_test.jl:19-56 end to end on the GPU."""
import math

import numpy as np
import pytest

import kpm_gb300 as kg
from kpm_gb300 import models
from oracle import ed_reference as ed
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _decaying_mu2d(rng, NC):
    n = np.arange(NC)
    env = np.exp(-(n[:, None] + n[None, :]) / (NC / 3))
    M = (rng.standard_normal((NC, NC)) + 1j * rng.standard_normal((NC, NC))) * env
    return (M + M.conj().T) / 2


@pytest.mark.parametrize("beta", [math.inf, 25.0])
def test_kubo_matches_oracle(beta):
    rng = np.random.default_rng(7)
    NC = 64
    mu = _decaying_mu2d(rng, NC)
    a, b = 3.1, 0.25
    Efs = np.linspace(-2.5, 2.5, 17)
    got = kg.kubo_bastin_cond(mu, a, Efs, b=b, NH=200, area=173.2, beta=beta)
    ref = np.array([ko.kubo_bastin_cond(mu, a, e, b=b, NH=200, area=173.2, beta=beta)
                    for e in Efs])
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(got - ref).max() <= 1e-11 * scale


def test_kubo_options_match_oracle():
    rng = np.random.default_rng(9)
    mu = _decaying_mu2d(rng, 80)
    kern = ko.lorentz_kernels(4.0)
    kw = dict(b=-0.1, NH=64, area=50.0, NC=70, quad_N=333, edge_cutoff=0.02)
    for e in (-1.0, 0.0, 0.4):
        got = kg.kubo_bastin_cond(mu, 1.7, e, kernel=kern, **kw)
        ref = ko.kubo_bastin_cond(mu, 1.7, e, kernel=kern, **kw)
        assert isinstance(got, float)
        assert abs(got - ref) <= 1e-11 * max(abs(ref), 1e-3)


def test_kubo_vector_equals_scalar_calls():
    rng = np.random.default_rng(2)
    mu = _decaying_mu2d(rng, 48)
    Efs = np.array([-0.7, 0.0, 0.3, 1.1])
    vec = kg.kubo_bastin_cond(mu, 2.0, Efs, NH=10, area=1.0)
    for e, v in zip(Efs, vec):
        assert kg.kubo_bastin_cond(mu, 2.0, float(e), NH=10, area=1.0) == v


def test_kubo_argument_errors():
    mu = np.eye(8, dtype=complex)
    for kw in (dict(NH=0, area=1.0), dict(NH=4, area=0.0), dict(NH=4, area=1.0, quad_N=0),
               dict(NH=4, area=1.0, edge_cutoff=1.0)):
        with pytest.raises(kg.KPMArgumentError):
            kg.kubo_bastin_cond(mu, 1.0, 0.0, **kw)
    with pytest.raises(kg.KPMArgumentError):
        kg.kubo_bastin_cond(mu, -1.0, 0.0, NH=4, area=1.0)


def test_haldane_hall_quantized_gpu_reconstruction():
    """sigma_xy = C from GPU moments and the GPU reconstruction, over a grid
    of Fermi energies in the gap, and equal to the oracle's reconstruction."""
    t2 = 0.2
    H, Jx, Jy, area = models.haldane(6, 6, t=1.0, t2=t2)
    D = H.shape[0]
    a, b, Hn = ko.normalizeH(H, center=True)
    psi = np.eye(D, dtype=complex)
    mu = kg.kpm_2d(Hn, Jx, Jy, 96, D, D, psi_in=psi)
    C = round(ed.chern_number_fhs(ed.haldane_bloch(t=1.0, t2=t2), Nk=30))
    s_ed = ed.ed_hall_conductivity_T0(H, Jx, Jy, area, 0.0)
    Efs = np.array([-0.3, 0.0, 0.3])
    got = kg.kubo_bastin_cond(mu, a, Efs, b=b, NH=D, area=area)
    ref = np.array([ko.kubo_bastin_cond(mu, a, e, b=b, NH=D, area=area) for e in Efs])
    assert np.abs(got - ref).max() <= 1e-10
    assert abs(got[1] - s_ed) < 0.03
    assert np.abs(got - C).max() < 0.05
    got_T = kg.kubo_bastin_cond(mu, a, 0.0, b=b, NH=D, area=area, beta=50.0)
    assert abs(got_T - got[1]) < 0.01


def test_dos_matches_oracle():
    rng = np.random.default_rng(4)
    NC = 256
    mu = rng.standard_normal(NC) * np.exp(-np.arange(NC) / 60)
    mu[0] = 1.0
    a, b = 2.3, 0.4
    E, rho = kg.dos(mu, a, b=b)
    E_ref, rho_ref = ko.dos(mu, a, b=b)
    assert np.array_equal(E, E_ref)
    assert np.abs(rho - rho_ref).max() <= 1e-12 * np.abs(rho_ref).max()
    # explicit grid with points outside |E - b| < a, truncated NC, Lorentz kernel
    Eg = np.linspace(-4, 4, 301)
    kern = ko.lorentz_kernels(3.0)
    _, r2 = kg.dos(mu, a, b=b, E_grid=Eg, NC=200, kernel=kern)
    _, r2_ref = ko.dos(mu, a, b=b, E_grid=Eg, NC=200, kernel=kern)
    assert np.abs(r2 - r2_ref).max() <= 1e-12 * np.abs(r2_ref).max()
    assert np.all(r2[np.abs(Eg - b) >= a] == 0)


def test_dos_sum_rule_ring():
    """test/frontend_test.jl:173-195: the reconstructed DOS integrates to mu_0 = 1."""
    N = 400
    H = (models.ring(N) / 2.2).tocsc()
    NC = 256
    psi = np.eye(N, dtype=complex)[:, ::4]
    mu = kg.kpm_1d(H, NC, psi.shape[1], psi_in=psi)
    E, rho = kg.dos(mu, 2.2, N_tilde=4000)
    integral = np.trapezoid(rho, E) if hasattr(np, "trapezoid") else np.trapz(rho, E)
    assert abs(integral - 1.0) < 0.02


def test_dos_argument_errors():
    with pytest.raises(kg.KPMArgumentError):
        kg.dos(np.ones((2, 2)), 1.0)
    with pytest.raises(kg.KPMArgumentError):
        kg.dos(np.ones(8), 1.0, E_grid=np.zeros(3), E_range=[0, 1])
    with pytest.raises(kg.KPMArgumentError):
        kg.dos(np.ones(8), 1.0, dE_order=5)
    with pytest.raises(kg.KPMArgumentError):
        kg.dos(np.ones(8), 1.0, dE_order=-1)
    with pytest.raises(kg.KPMArgumentError):
        kg.dos0(np.ones(8), 1.0, dE_order=1)


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_dos_energy_derivatives_match_oracle(order):
    """dos(mu, a; dE_order) (src/applications/dos.jl:128-139): the device jets
    against the oracle's jets through cos(n acos x) (the arithmetic of the
    reference's nested ForwardDiff), and against finite differences of the
    dE_order - 1 curve."""
    rng = np.random.default_rng(40 + order)
    NC = 200
    mu = rng.standard_normal(NC) * np.exp(-np.arange(NC) / 50)
    mu[0] = 1.0
    a, b = 1.7, 0.35
    Eg = b + a * np.linspace(-0.97, 0.97, 41)
    Eg = np.concatenate([Eg, [b - 1.5 * a, b + 1.01 * a]])   # outside: zero
    _, d = kg.dos(mu, a, b=b, E_grid=Eg, dE_order=order)
    ref = ko.dos_derivative(mu, a, b, Eg, order)
    assert np.abs(d - ref).max() <= 1e-10 * np.abs(ref).max()
    assert np.all(d[-2:] == 0)
    h = 1e-5 * a
    E_in = Eg[:-2]
    _, up = kg.dos(mu, a, b=b, E_grid=E_in + h, dE_order=order - 1)
    _, dn = kg.dos(mu, a, b=b, E_grid=E_in - h, dE_order=order - 1)
    fd = (up - dn) / (2 * h)
    assert np.abs(d[:-2] - fd).max() <= 1e-5 * np.abs(fd).max()


def test_dos_derivative_reference_cases():
    """test/dos_test.jl:143-193: dE_order = 1 against central differences
    (rtol 1e-5), dE_order = 2 against the five-point stencil (rtol 1e-7) and
    against dos0 at the band centre (rtol 1e-10)."""
    rng = np.random.default_rng(23)
    NC, a, b = 48, 1.7, 0.35
    mu = rng.standard_normal(NC)
    E_grid = b + a * np.array([-0.45, 0.2, 0.55])
    h = 1e-3 * a

    def rho0(E):
        return kg.dos(mu, a, b=b, E_grid=[E], N_tilde=1)[1][0]

    stencil = np.array([(-rho0(E + 2 * h) + 16 * rho0(E + h) - 30 * rho0(E)
                         + 16 * rho0(E - h) - rho0(E - 2 * h)) / (12 * h * h) for E in E_grid])
    _, d2 = kg.dos(mu, a, b=b, E_grid=E_grid, N_tilde=3, dE_order=2)
    assert np.allclose(d2, stencil, rtol=1e-7, atol=0)
    _, d2c = kg.dos(mu, a, b=b, E_grid=[b], N_tilde=1, dE_order=2)
    assert abs(d2c[0] - kg.dos0(mu, a, dE_order=2)) <= 1e-10 * abs(d2c[0])
    assert abs(kg.dos0(mu, a) - kg.dos(mu, a, b=b, E_grid=[b])[1][0]) <= 1e-10 * abs(kg.dos0(mu, a))
    h1 = 1e-4 * a
    _, d1 = kg.dos(mu, a, b=b, E_grid=E_grid, dE_order=1)
    fd = (kg.dos(mu, a, b=b, E_grid=E_grid + h1)[1] - kg.dos(mu, a, b=b, E_grid=E_grid - h1)[1]) / (2 * h1)
    assert np.allclose(d1, fd, rtol=1e-5, atol=0)

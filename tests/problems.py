"""Seeded problem generators shared by the CPU and GPU tests.

Arrays are numpy float64 in the mlgpu.h layout.  Values are chosen so every
closure regime (solid, eutectic, mush, liquid) appears.
"""
import numpy as np

from mushy_gb300 import abi


def grid(n, periodic=(0, 0, 0)):
    return abi.make_grid(list(n), 1.0 / n[0], periodic)


def mushy_params(**kw):
    base = dict(stefan=5.0, compositionRatio=5.0, waterDistributionCoeff=1e-3,
                specificHeatRatio=1.0)
    base.update(kw)
    return abi.make_params(**base)


def hc_state(g, rng, regimes=True):
    """(H, C) covering solid/eutectic/mush/liquid for St=5, CR=5."""
    shape = (1,) + abi.cell_shape(g)
    phi = np.empty((2,) + abi.cell_shape(g))
    if regimes:
        phi[0] = rng.uniform(-0.5, 7.0, abi.cell_shape(g))
        phi[1] = rng.uniform(-4.0, -0.5, abi.cell_shape(g))
    else:
        phi[0] = 6.0 + 0.01 * rng.standard_normal(abi.cell_shape(g))
        phi[1] = -1.0 + 0.01 * rng.standard_normal(abi.cell_shape(g))
    return phi


def faces(g, rng, ncomp, lo=0.5, hi=1.5, sign=-1.0):
    return [sign * rng.uniform(lo, hi, (ncomp,) + abi.face_shape(g, d)) for d in range(g.dim)]


def hc_bcs(kind="mixed"):
    """phi BC = no flux; derived BC: Dirichlet T/C_l on y, Neumann on x."""
    phi_bc = abi.make_bc()
    if kind == "neumann":
        return phi_bc, abi.make_bc()
    spec = {(1, 0, 0): (abi.BC_DIRICHLET, -1.0), (1, 1, 0): (abi.BC_DIRICHLET, 0.5),
            (1, 0, 1): (abi.BC_DIRICHLET, -1.0), (1, 1, 1): (abi.BC_DIRICHLET, -1.0),
            (0, 0, 0): (abi.BC_NEUMANN, 0.3), (0, 1, 1): (abi.BC_NEUMANN, -0.2),
            (2, 0, 0): (abi.BC_DIRICHLET, 0.25), (2, 1, 1): (abi.BC_NEUMANN, 0.1)}
    return phi_bc, abi.make_bc(spec)


def temperature_bcs(method=0, max_iter=2, limit=0.0, dim=2):
    """Temperature conditions on H (C no flux), derived BC unused:
    x lo fixed temperature, x hi temperature flux, y lo radiation (with a
    no-flux limit along x), y hi no flux; z lo fixed temperature in 3D."""
    spec = {(0, 0, 0): (abi.BC_FIXED_TEMPERATURE, -0.4),
            (0, 1, 0): (abi.BC_TEMPERATURE_FLUX, 0.8),
            (1, 0, 0): (abi.BC_TEMPERATURE_FLUX_RADIATION, -0.3),
            (1, 1, 0): (abi.BC_NEUMANN, 0.0)}
    if dim == 3:
        spec[(2, 0, 0)] = (abi.BC_FIXED_TEMPERATURE, 0.6)
    nlbc = abi.make_nlbc(radiation={(1, 0): (0.7, 1.3, -1.2)},
                         no_flux_limit={(1, 0): limit}, method=method, max_iter=max_iter)
    return abi.make_bc(spec), abi.make_bc(), nlbc


def vc_bc(kind="mixed"):
    if kind == "neumann":
        return abi.make_bc()
    spec = {(0, 0, 0): (abi.BC_DIRICHLET, 0.7), (0, 1, 0): (abi.BC_NEUMANN, -0.4),
            (1, 0, 0): (abi.BC_NEUMANN, 0.2), (1, 1, 0): (abi.BC_DIRICHLET, -0.3),
            (2, 0, 0): (abi.BC_DIRICHLET, 0.1), (2, 1, 0): (abi.BC_NEUMANN, 0.05)}
    return abi.make_bc(spec)


def smooth_field(shape, rng, sigma):
    """Gaussian-filtered white noise (FFT, periodic), unit std."""
    w = rng.standard_normal(shape)
    k = [np.fft.fftfreq(n) for n in shape]
    kk = np.meshgrid(*k, indexing="ij")
    filt = np.exp(-2 * np.pi ** 2 * sigma ** 2 * sum(x ** 2 for x in kk))
    f = np.real(np.fft.ifftn(np.fft.fftn(w) * filt))
    return (f - f.mean()) / f.std()


def projection_problem(n, seed, sigma=32.0):
    """Config-2-style problem: Kozeny-Carman permeability of a smooth random
    porosity in [0.05, 1], capped at 1e4; rhs = div of a random face velocity
    with the mean removed; periodic in x, Neumann in y."""
    rng = np.random.default_rng(seed)
    dim = len(n)
    g = abi.make_grid(list(n), 1.0 / n[0], (1, 0, 0))
    shape = abi.cell_shape(g)
    f = smooth_field(shape[-dim:], rng, sigma if sigma < min(n) else min(n) / 4)
    f = (f - f.min()) / (f.max() - f.min())
    chi = 0.05 + 0.95 * f
    chi = chi.reshape(shape)
    with np.errstate(divide="ignore"):
        perm = np.where(chi < 1.0, chi ** 3 / np.maximum((1 - chi) ** 2, 1e-300), 1e4)
    perm = np.minimum(perm, 1e4)
    u = [rng.standard_normal(abi.face_shape(g, d)) for d in range(dim)]
    return g, chi, perm, u

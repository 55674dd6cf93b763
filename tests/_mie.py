"""Mie series for a perfectly conducting sphere (test helper): the surface current J = n x H of
an incident plane wave E_inc = x_hat exp(i kappa z) (time factor exp(-i omega t), mu = eps = 1,
omega = kappa), from the published vector-spherical-wave expansion (Bohren and Huffman,
Absorption and Scattering of Light by Small Particles, ch. 4: the incident expansion 4.37, the
wave functions 4.50, the angular functions pi_n, tau_n of 4.46-4.47, and the coefficients of
the conducting limit a_n = psi_n' / xi_n', b_n = psi_n / xi_n with psi_n = x j_n, xi_n = x h_n).
For that current the electric-field integral equation reads i (V J, v) = -(E_inc, v) with V the
Maxwell single layer kappa <u, v> G - 1/kappa <div u, div v> G."""
import numpy as np
from scipy.special import spherical_jn, spherical_yn


def mie_current(points, radius, kappa, nmax=None):
    """J = n x (H_inc + H_scat) on the sphere at the directions of points (np, 3): (np, 3) complex."""
    P = np.asarray(points, dtype=np.float64)
    r = np.linalg.norm(P, axis=1)
    theta = np.arccos(np.clip(P[:, 2] / r, -1.0, 1.0))
    phi = np.arctan2(P[:, 1], P[:, 0])
    x = kappa * radius
    N = nmax or int(x + 4.0 * x ** (1.0 / 3.0) + 8)
    mu = np.cos(theta)
    # angular functions: pi_0 = 0, pi_1 = 1, pi_n = (2n-1)/(n-1) mu pi_{n-1} - n/(n-1) pi_{n-2};
    # tau_n = n mu pi_n - (n+1) pi_{n-1}
    pis = [np.zeros_like(mu), np.ones_like(mu)]
    for n in range(2, N + 1):
        pis.append((2 * n - 1) / (n - 1) * mu * pis[n - 1] - n / (n - 1) * pis[n - 2])
    Hth = np.zeros_like(mu, dtype=complex)
    Hph = np.zeros_like(mu, dtype=complex)
    for n in range(1, N + 1):
        pi_n, tau_n = pis[n], n * mu * pis[n] - (n + 1) * pis[n - 1]
        jn, jd = spherical_jn(n, x), spherical_jn(n, x, derivative=True)
        yn, yd = spherical_yn(n, x), spherical_yn(n, x, derivative=True)
        hn, hd = jn + 1j * yn, jd + 1j * yd
        psi, dpsi = x * jn, jn + x * jd
        xi, dxi = x * hn, hn + x * hd
        an, bn = dpsi / dxi, psi / xi
        En = 1j ** n * (2 * n + 1) / (n * (n + 1))
        # H = -sum E_n (M_e1n^(1) + i N_o1n^(1)) + sum E_n (i b_n N_o1n^(3) + a_n M_e1n^(3)); the
        # tangential parts at rho = x: M_e1n: (-sin phi pi_n, -cos phi tau_n) z_n, N_o1n:
        # (sin phi tau_n, cos phi pi_n) [rho z_n]' / rho
        cm = (-psi + an * xi) / x
        cn = 1j * (bn * dxi - dpsi) / x
        Hth += En * (cm * (-np.sin(phi) * pi_n) + cn * (np.sin(phi) * tau_n))
        Hph += En * (cm * (-np.cos(phi) * tau_n) + cn * (np.cos(phi) * pi_n))
    eth = np.stack([np.cos(theta) * np.cos(phi), np.cos(theta) * np.sin(phi), -np.sin(theta)], 1)
    eph = np.stack([-np.sin(phi), np.cos(phi), np.zeros_like(phi)], 1)
    # n x H with n = e_r: e_r x e_theta = e_phi, e_r x e_phi = -e_theta
    return Hth[:, None] * eph - Hph[:, None] * eth

"""Independent restatements of the reference's fall-speed and ice-shape functions,
shared by the oracle tests (test_oracle.py) and the sedimentation tests
(test_sedim.py): terminal_vel's liquid regimes and its Khvorostyanov-Curry ice
branch (src/src_shared/mo_particle_external_properties.f90:43-158), and
getShapeCoefficients / getDiameter (src/src_shared/mo_ice_shape.f90:46-191)."""
import math


def terminal_vel_numpy(d, rhop, rhoa, visc, beta):
    """Independent restatement of the liquid regimes of terminal_vel
    (src/src_shared/mo_particle_external_properties.f90:43-100): Stokes with the
    Cunningham factor below 19 um, Beard's Davies-number fit up to 1.07 mm, the Bond-number
    fit above, capped at 9.2 m/s."""
    grav, surfw0 = 9.81, 0.073
    if d <= 19e-6:
        return d * d * (rhop - rhoa) * grav * beta / (18. * visc)
    if d < 1.07e-3:
        nda = 4. / 3. * d ** 3. * grav * (rhop - rhoa) * rhoa / visc ** 2.
        x = math.log(nda)
        y = (-0.318657e1 + 0.992696 * x - 0.153193e-2 * x ** 2 - 0.987059e-3 * x ** 3
             - 0.578878e-3 * x ** 4 + 0.855176e-4 * x ** 5 - 0.327815e-5 * x ** 6)
        return visc / rhoa / d * (beta * math.exp(y))
    npn = surfw0 ** 3. * rhoa ** 2. / (visc ** 4. * (rhop - rhoa) * grav)
    bo = 4. / 3. * (rhop - rhoa) * grav / surfw0 * d ** 2.
    x3 = math.log(bo * npn ** (1. / 6.))
    y3 = (-0.500015e1 + 0.523778e1 * x3 - 0.204914e1 * x3 ** 2 + 0.475294 * x3 ** 3
          - 0.542819e-1 * x3 ** 4 + 0.238449e-2 * x3 ** 5)
    return min(visc / rhoa / d * (npn ** (1. / 6.) * math.exp(y3)), 9.2)


RHO_IC, RHO_RI = 917., 400.
ICE_A, ICE_B, ICE_G, ICE_S = 15.56999e-3, 2.02, 0.55, 1.97


def ice_shape_numpy(mpri, mrim, numc):
    """Independent restatement of getShapeCoefficients and getDiameter
    (src/src_shared/mo_ice_shape.f90:46-91, 104-141, 145-191) for the default
    Khvorostyanov-Curry crystal coefficients: returns (alpha, beta, gamma, sigma), the
    maximum dimension and the regime (0 spherical ice, 1 dense non-spherical, 2 graupel,
    3 partially rimed).  The rime fraction is clipped to [1e-4, 0.9999] and the bulk
    density is rime-weighted, so the regime limits move with the rime fraction."""
    pi, pi6 = 3.1415927, 0.5235988
    sph = (pi6 * RHO_IC, 3., pi / 4., 2.)
    if numc < 1.e-6:
        return sph, 1.e-9, -1
    m = (mpri + mrim) / numc                              # mass of one particle
    fr = max(min(mrim / (m * numc), 0.9999), 0.0001)
    rho_b = fr * RHO_RI + (1. - fr) * RHO_IC
    # m = alpha D^beta meets the spheres of density rhoic, rho_b, rho_b/(1-fr)
    d_th = (pi6 * RHO_IC / ICE_A) ** (1. / (ICE_B - 3.))
    d_gr = (ICE_A / (pi6 * rho_b)) ** (1. / (3. - ICE_B))
    d_cr = (ICE_A / (1. - fr) / (pi6 * rho_b)) ** (1. / (3. - ICE_B))
    m_th = RHO_IC * pi6 * d_th * d_th * d_th
    m_gr = rho_b * pi6 * d_gr * d_gr * d_gr
    m_cr = rho_b * pi6 * d_cr * d_cr * d_cr
    if m < m_th:
        return sph, (m / (pi6 * RHO_IC)) ** (1. / 3.), 0
    if m < m_gr:
        return (ICE_A, ICE_B, ICE_G, ICE_S), (m / ICE_A) ** (1. / ICE_B), 1
    if m < m_cr:
        return sph, (m / (pi6 * rho_b)) ** (1. / 3.), 2
    coeffs = sph if m == m_cr else (ICE_A / (1. - fr), ICE_B, ICE_G * (1. - fr) + pi / 4. * fr,
                                    ICE_S * (1. - fr) + 2. * fr)
    return coeffs, (m * (1. - fr) / ICE_A) ** (1. / ICE_B), 3


def ice_terminal_vel_numpy(dsph, dmax, rhop, rhoa, visc, shape):
    """Independent restatement of the ice branch of terminal_vel
    (src/src_shared/mo_particle_external_properties.f90:88-96, 103-158): the power law
    V = A_v D^B_v of Khvorostyanov and Curry (2002) eqs. 2.12-2.13 and 2.23-2.25, with the
    Best number X formed from the spherical-equivalent volume and the area gamma D^sigma
    of the maximum dimension D."""
    grav, c1, delta0 = 9.81, 0.0902, 9.06
    alpha, beta, gamma, sigma = shape
    vb = 0.5235988 * dsph * dsph * dsph
    area = gamma * dmax ** sigma
    x = 2. * vb * (rhop - rhoa) * grav * dmax * dmax / (area * rhoa * visc * visc)
    s = math.sqrt(1. + c1 * math.sqrt(x))
    b_re = 0.5 * c1 * math.sqrt(x) / ((s - 1.) * s)
    a_re = 0.25 * delta0 * delta0 * (s - 1.) * (s - 1.) / x ** b_re
    a_v = a_re * visc ** (1. - 2. * b_re) * (2. * alpha * grav / (rhoa * gamma)) ** b_re
    b_v = b_re * (beta - sigma + 2.) - 1.
    return a_v * dmax ** b_v

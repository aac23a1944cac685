"""CPU: the reduced-precision MRT operators are the reference's MRT.

* The deviation-form MRT of the FP32/16-bit kernels (collide_bulk_dev, model
  3) equals the reference's moment-space MRT (serial/CellFunctions.c:401-438
  with MRTInitializer's relaxation rates, serial/CellFunctions.c:60-90) applied
  to f = d + w rho0; likewise BGK and TRT (serial/CellFunctions.c:352-395; the
  reference's float rounding of the TRT split terms is kept by the FP64 path
  only, so the comparison here is in exact arithmetic).
* The folded-constant operator of the two-node 16-bit kernel
  (collide_mrt_pair_raw: raw stored values in and out) equals the
  deviation-form one.
* The moment storage's bulk step (lbm_mom.cuh): its decode with folded
  constants is the reference transform's inverse, and its collision folded
  into the encoding is the reference's MRT relaxation.
Each is restated here in float64 from its source."""
import numpy as np

C36W = np.array([16, 4, 4, 4, 4, 1, 1, 1, 1], float)  # 36 w_k


def mrt_dev(F, rho0, om):
    """collide_bulk_dev<3>: deviations d_k = f_k - w_k rho0 in and out."""
    a13, a24 = F[1] + F[3], F[2] + F[4]
    a14 = a13 + a24
    p57, p68 = F[5] + F[7], F[6] + F[8]
    a58 = p57 + p68
    rt = (F[0] + a14) + a58
    rho = rho0 + rt
    m1 = 2 * a58 - a14 - 4 * F[0]
    m2 = (4 * F[0] + a58) - 2 * a14
    d13, d24 = F[1] - F[3], F[2] - F[4]
    e57, e86 = F[5] - F[7], F[8] - F[6]
    x58, y58 = e57 + e86, e57 - e86
    jx, jy = d13 + x58, d24 + y58
    m4, m6 = x58 - 2 * d13, y58 - 2 * d24
    m7, m8 = a13 - a24, p57 - p68
    inv = 1 / rho
    jj = jx * jx + jy * jy
    d1 = 1.4 * (m1 + 2 * rt - 3 * jj)
    d2 = 1.4 * (m2 - rt + 3 * jj)
    d4 = 1.2 * (m4 + jx)
    d6 = 1.2 * (m6 + jy)
    d7 = om * (m7 - (jx * jx - jy * jy) * inv)
    d8 = om * (m8 - jx * jy * inv)
    c = 1 / 36
    ax, dg = -d1 - 2 * d2, 2 * d1 + d2
    X, Y, P = -6 * d4, -6 * d6, 9 * d7
    Xd, Yd, Q = 3 * d4, 3 * d6, 9 * d8
    return np.array([
        F[0] - c * (4 * (d2 - d1)),
        F[1] - c * (ax + X + P), F[2] - c * (ax + Y - P),
        F[3] - c * (ax - X + P), F[4] - c * (ax - Y - P),
        F[5] - c * (dg + Xd + Yd + Q), F[6] - c * (dg - Xd + Yd - Q),
        F[7] - c * (dg - Xd - Yd + Q), F[8] - c * (dg + Xd - Yd - Q)])


def mrt_raw(S, rho0, om, u0):
    """collide_mrt_pair_raw: stored values s_k = d_k / (36 w_k u0) in and out."""
    t13, t24 = S[1] + S[3], S[2] + S[4]
    t14 = t13 + t24
    p57, p68 = S[5] + S[7], S[6] + S[8]
    a58 = p57 + p68
    rt = 16 * S[0] + (4 * t14 + a58)
    rho = u0 * rt + rho0
    u13, u24 = S[1] - S[3], S[2] - S[4]
    e57, e86 = S[5] - S[7], S[8] - S[6]
    x58, y58 = e57 + e86, e57 - e86
    jx, jy = 4 * u13 + x58, 4 * u24 + y58
    E4, E6 = -2 * u13 + x58, -2 * u24 + y58
    w7, m8 = t13 - t24, p57 - p68
    jj = jx * jx + jy * jy
    ninv = -u0 / rho
    g1 = -3 * u0 * jj + (-32 * S[0] + 4 * (a58 + t14))
    g2 = 3 * u0 * jj + (48 * S[0] - 12 * t14)
    h7 = (jx - jy) * (jx + jy) * ninv + 4 * w7
    h8 = jx * jy * ninv + m8
    P4, Q = om / 16 * h7, 0.25 * om * h8
    A4 = -1.4 / 144 * (2 * g2 + g1)
    D = 1.4 / 36 * (2 * g1 + g2)
    ApP, AmP, DpQ, DmQ = A4 + P4, A4 - P4, D + Q, D - Q
    S46, T46 = E4 + E6, E4 - E6
    return np.array([
        -5.6 / 576 * (g2 - g1) + S[0],
        0.1 * E4 + (S[1] - ApP), 0.1 * E6 + (S[2] - AmP),
        -0.1 * E4 + (S[3] - ApP), -0.1 * E6 + (S[4] - AmP),
        -0.2 * S46 + (S[5] - DpQ), 0.2 * T46 + (S[6] - DmQ),
        0.2 * S46 + (S[7] - DpQ), -0.2 * T46 + (S[8] - DmQ)])


# the reference's MRT transform and its inverse (x 36), serial/CellFunctions.c:24-47
TM = np.array([[1, 1, 1, 1, 1, 1, 1, 1, 1], [-4, -1, -1, -1, -1, 2, 2, 2, 2],
               [4, -2, -2, -2, -2, 1, 1, 1, 1], [0, 1, 0, -1, 0, 1, -1, -1, 1],
               [0, -2, 0, 2, 0, 1, -1, -1, 1], [0, 0, 1, 0, -1, 1, 1, -1, -1],
               [0, 0, -2, 0, 2, 1, 1, -1, -1], [0, 1, -1, 1, -1, 0, 0, 0, 0],
               [0, 0, 0, 0, 0, 1, -1, 1, -1]], float)
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], float)
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], float)


def mrt_reference(f, om):
    """Moment-space MRT on absolute populations: f - Minv S (M f - m_eq)."""
    R = f.sum(0)
    U, V = (CX[:, None] * f).sum(0) / R, (CY[:, None] * f).sum(0) / R
    meq = np.array([R, R * (-2 + 3 * R * (U * U + V * V)), R * (1 - 3 * R * (U * U + V * V)),
                    R * U, -R * U, R * V, -R * V, R * (U * U - V * V), R * U * V])
    S = np.diag([1.0, 1.4, 1.4, 1.0, 1.2, 1.0, 1.2, om, om])
    return f - np.linalg.inv(TM) @ S @ (TM @ f - meq)


def test_deviation_operator_equals_reference_mrt():
    rng = np.random.default_rng(3)
    w = C36W / 36
    for rho0 in (1.0, 5.0):
        for om in (1.9, 1.1):
            d = w[:, None] * rho0 * rng.normal(0, 0.3, (9, 400))
            f = d + w[:, None] * rho0
            ref = mrt_reference(f, om) - w[:, None] * rho0
            got = mrt_dev(d, rho0, om)
            assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


OPP = [0, 3, 4, 1, 2, 7, 8, 5, 6]


def feq_abs(f):
    R = f.sum(0)
    U, V = (CX[:, None] * f).sum(0) / R, (CY[:, None] * f).sum(0) / R
    w = C36W / 36
    cu = CX[:, None] * U + CY[:, None] * V
    return R * w[:, None] * (1 + 3 * cu + 4.5 * cu ** 2 - 1.5 * (U * U + V * V))


def bgk_trt_dev(F, rho0, om, omA, model):
    """collide_bulk_dev, models 1 (BGK) and 2 (TRT), on deviations."""
    rt = F.sum(0)
    jx, jy = (CX[:, None] * F).sum(0), (CY[:, None] * F).sum(0)
    rho = rho0 + rt
    u, v = jx / rho, jy / rho
    w = C36W / 36
    T2 = CX[:, None] * u + CY[:, None] * v
    feq = w[:, None] * (rt + rho * (3 * T2 + 4.5 * T2 * T2 - 1.5 * (u * u + v * v)))
    if model == 1:
        return om * (feq - F) + F
    sp = 0.5 * ((F + F[OPP]) - (feq + feq[OPP]))
    sm = 0.5 * ((F - F[OPP]) - (feq - feq[OPP]))
    return F - om * sp - omA * sm


def test_deviation_bgk_trt_equal_reference():
    rng = np.random.default_rng(11)
    w = C36W / 36
    for rho0 in (1.0, 5.0):
        om = 1.7
        omA = 8 * (2 - om) / (8 - om)  # serial/Iterate.c:180
        d = w[:, None] * rho0 * rng.normal(0, 0.3, (9, 400))
        f = d + w[:, None] * rho0
        fe = feq_abs(f)
        bgk = om * fe + (1 - om) * f
        trt = f - 0.5 * ((f + f[OPP]) - (fe + fe[OPP])) * om - 0.5 * ((f - f[OPP]) - (fe - fe[OPP])) * omA
        for model, ref in ((1, bgk), (2, trt)):
            got = bgk_trt_dev(d, rho0, om, omA, model) + w[:, None] * rho0
            assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), model


def test_folded_raw_operator_equals_deviation_operator():
    rng = np.random.default_rng(7)
    for rho0 in (1.0, 2.5):
        for S_scale in (4096.0, 1.0):  # FP16 and BF16 scales
            u0 = rho0 / (36 * S_scale)
            for om in (1.9, 1.2):
                w = C36W / 36
                # deviations of a flow with |u| ~ 0.1 and small non-equilibrium parts
                d = w[:, None] * rho0 * rng.normal(0, 0.3, (9, 500))
                ref = mrt_dev(d, rho0, om)
                s = d / (C36W[:, None] * u0)
                got = mrt_raw(s, rho0, om, u0) * (C36W[:, None] * u0)
                assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


# ---- moment storage (LBM_FP16NEQ): parallellbmcranfield_gb300/csrc/lbm_mom.cuh
# A node's stored set is r = rho - rho0, j = (x, y) and six non-equilibrium
# moments n_i (stored units: n_i = S (m_i - b_i), S = 4096) of the rows 1, 2,
# 4, 6, 7, 8 of the reference's transform applied to d_k = f_k - w_k rho0;
# b_1 = -2 r + 3 |j|^2, b_2 = r - 3 |j|^2, b_4 = -x, b_6 = -y,
# b_7 = (x^2 - y^2) / rho0, b_8 = x y / rho0.
MOM_S = 4096.0


def mom_refs(r, x, y, rho0):
    jj = x * x + y * y
    return np.array([-2 * r + 3 * jj, r - 3 * jj, -x, -y, (x * x - y * y) / rho0, x * y / rho0])


def mom_decode_folded(r, x, y, n, rho0):
    """mom_decode2: populations of a stored set with the 1/36 of the inverse
    transform and the storage scale folded into the constants."""
    s = 1 / MOM_S
    yy = y * y
    jj = x * x + yy
    xmy = jj - 2 * yy
    i4 = 0.25 / rho0
    dg = n[1] * (s / 36) + (n[0] * (2 * s / 36) + (jj / 12 + r / 36))
    Q = n[5] * (s / 4) + x * y * i4
    Xd, Yd = n[2] * (s / 12) + x / 12, n[3] * (s / 12) + y / 12
    gp, gm, sp, sm = dg + Q, dg - Q, Xd + Yd, Xd - Yd
    d5, d6, d7, d8 = gp + sp, gm - sm, gp - sp, gm + sm
    ax = n[1] * (-2 * s / 36) + (n[0] * (-s / 36) + (jj * 3 / 36 + r * 4 / 36))
    P = n[4] * (s / 4) + xmy * i4
    s13, s24 = ax + P, ax - P
    e57, e86 = d5 - d7, d8 - d6
    dx, dy = x - (e57 + e86), y - (e57 - e86)
    d1, d3, d2, d4 = 0.5 * dx + s13, -0.5 * dx + s13, 0.5 * dy + s24, -0.5 * dy + s24
    d0 = r - (((d1 + d3) + (d2 + d4)) + ((d5 + d7) + (d6 + d8)))
    return np.array([d0, d1, d2, d3, d4, d5, d6, d7, d8])


def test_moment_decode_is_the_inverse_transform():
    """The folded decode returns Minv m for m = (r, b_1 + n_1/S, b_2 + n_2/S, x,
    b_4 + n_4/S, y, b_6 + n_6/S, b_7 + n_7/S, b_8 + n_8/S)."""
    rng = np.random.default_rng(21)
    Minv = np.linalg.inv(TM)
    for rho0 in (1.0, 5.0):
        r = rho0 * rng.normal(0, 0.02, 300)
        x, y = rho0 * rng.normal(0, 0.05, (2, 300))
        n = MOM_S * rho0 * rng.normal(0, 1e-3, (6, 300))
        b = mom_refs(r, x, y, rho0)
        m = b + n / MOM_S
        mv = np.array([r, m[0], m[1], x, m[2], y, m[3], m[4], m[5]])
        ref = Minv @ mv
        got = mom_decode_folded(r, x, y, n, rho0)
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
        # and the transform of the decoded populations gives the set back
        back = TM @ got
        assert np.abs(back[[0, 3, 5]] - np.array([r, x, y])).max() <= 1e-13 * rho0


def test_moment_collision_folded_into_the_encoding():
    """mom_collide_store2: n_i = S (1 - s_i) m_i + S s_i e_i - S b_i equals
    S (m_i - s_i (m_i - e_i) - b_i), the reference's MRT relaxation of the pulled
    moments (serial/CellFunctions.c:401-438: rates 1.4, 1.4, 1.2, 1.2, omega,
    omega; e_1 = -2 r + 3 |j|^2, e_2 = r - 3 |j|^2, e_4 = -x, e_6 = -y,
    e_7 = (x^2 - y^2) / rho, e_8 = x y / rho) stored against the references of
    the (rounded) stored r, j; checked against the moment-space operator of
    mrt_reference on f = d + w rho0."""
    rng = np.random.default_rng(22)
    w = C36W / 36
    for rho0 in (1.0, 2.5):
        for om in (1.9, 1.3):
            d = w[:, None] * rho0 * rng.normal(0, 0.3, (9, 400))
            mom = TM @ d  # pulled moments of the deviations
            r, x, y = mom[0], mom[3], mom[5]
            m = mom[[1, 2, 4, 6, 7, 8]]
            rho = rho0 + r
            jj = x * x + y * y
            e = np.array([-2 * r + 3 * jj, r - 3 * jj, -x, -y, (x * x - y * y) / rho, x * y / rho])
            s = np.array([1.4, 1.4, 1.2, 1.2, om, om])[:, None]
            # the stored r, j after rounding to the 24-bit grid
            rq = np.round(r * 2 ** 24) / 2 ** 24
            xq, yq = np.round(x * 2 ** 25) / 2 ** 25, np.round(y * 2 ** 25) / 2 ** 25
            b = mom_refs(rq, xq, yq, rho0)
            folded = MOM_S * (1 - s) * m + MOM_S * s * e - MOM_S * b
            direct = MOM_S * (m - s * (m - e) - b)
            assert np.abs(folded - direct).max() <= 1e-10 * np.abs(direct).max()
            # the post-collision moments are the reference operator's
            f = d + w[:, None] * rho0
            post = TM @ (mrt_reference(f, om) - w[:, None] * rho0)
            assert np.abs(post[[1, 2, 4, 6, 7, 8]] - (m - s * (m - e))).max() <= 1e-12 * rho0

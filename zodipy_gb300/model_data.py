"""Published parameter sets of the built-in zodiacal light models.

These are physical model constants, not code: the Kelsall et al. (1998)
DIRBE fit, the Planck 2013/2015/2018 and Odegard et al. (2019) emissivity
refits, and the Rowan-Robinson & May (2013) model.  They must equal the values
the reference ships (``zodipy/component_params.py:19-204``,
``zodipy/source_params.py:5-271``) so
that outputs agree; ``tests/test_model_data.py`` checks them against a dump of
the reference's own registry.
"""

from __future__ import annotations

from .components import (
    Band,
    BroadBand,
    Cloud,
    Comet,
    ComponentLabel,
    Fan,
    Feature,
    FeatureRRM,
    Interstellar,
    NarrowBand,
    Ring,
    RingRRM,
)

L = ComponentLabel

# Kelsall et al. (1998) Table 1 geometry, as fitted to DIRBE.
DIRBE_COMPONENTS = {
    L.CLOUD: (
        Cloud,
        dict(
            x_0=0.011887800744346281,
            y_0=0.005476506466226378,
            z_0=-0.0021530908020710744,
            i=2.033518807239077,
            Omega=77.65795555409711,
            n_0=1.134437388142796e-07,
            alpha=1.337069670593028,
            beta=4.141500415758664,
            gamma=0.9420617939335804,
            mu=0.1887317648909019,
        ),
    ),
    L.BAND1: (
        Band,
        dict(
            x_0=0.0,
            y_0=0.0,
            z_0=0.0,
            i=0.5643826515438973,
            Omega=80.0,
            n_0=5.589029040322837e-10,
            delta_zeta=8.785053440871303,
            v=0.10000000149011612,
            p=4.0,
            delta_r=1.5,
        ),
    ),
    L.BAND2: (
        Band,
        dict(
            x_0=0.0,
            y_0=0.0,
            z_0=0.0,
            i=1.2000000476837158,
            Omega=30.347475578624532,
            n_0=1.98776094225908e-09,
            delta_zeta=1.991703242577764,
            v=0.8999999761581421,
            p=4.0,
            delta_r=0.9412188120165115,
        ),
    ),
    L.BAND3: (
        Band,
        dict(
            x_0=0.0,
            y_0=0.0,
            z_0=0.0,
            i=0.800000011920929,
            Omega=80.0,
            n_0=1.4369827283512384e-10,
            delta_zeta=15.0,
            v=0.05000000074505806,
            p=4.0,
            delta_r=1.5,
        ),
    ),
    L.RING: (
        Ring,
        dict(
            x_0=0.0,
            y_0=0.0,
            z_0=0.0,
            i=0.4870716600681924,
            Omega=22.278979678854448,
            n_0=1.8260527826501675e-08,
            R=1.0281924326308751,
            sigma_r=0.02500000037252903,
            sigma_z=0.0540680373569781,
        ),
    ),
    L.FEATURE: (
        Feature,
        dict(
            x_0=0.0,
            y_0=0.0,
            z_0=0.0,
            i=0.4870716600681924,
            Omega=22.278979678854448,
            n_0=2.0094267183590947e-08,
            R=1.0579182694524214,
            sigma_r=0.10287314662396611,
            sigma_z=0.09144296376871602,
            theta=-10.0,
            sigma_theta=12.11521093393874,
        ),
    ),
}

# The Planck refits drop the ring and the feature.
PLANCK_COMPONENTS = {k: v for k, v in DIRBE_COMPONENTS.items() if k not in (L.RING, L.FEATURE)}

T_0_DIRBE = 286.0
DELTA_DIRBE = 0.46686259861486573

DIRBE_BANDS_MICRON = [1.25, 2.2, 3.5, 4.9, 12.0, 25.0, 60.0, 100.0, 140.0, 240.0]
IRAS_BANDS_MICRON = [12.0, 25.0, 60.0, 100.0]

# Rowan-Robinson & May (2013): geometry (component_params.py:98-204), grain temperatures
# (source_params.py:7-31) and the per-band calibration (source_params.py:37-39).
R_MARS = 1.5237
R_ASTEROID_BELT = 3.137
R_KUIPER_BELT = 30.0
_RRM_PLANE = dict(x_0=0.0, y_0=0.0, z_0=0.0, i=1.5, Omega=78.0)
RRM_COMPONENTS = {
    L.FAN: (Fan, dict(_RRM_PLANE, P=2.13, Q=10.7, gamma=1.3, Z_0=0.06, R_outer=R_MARS)),
    L.COMET: (Comet, dict(_RRM_PLANE, P=2.5, gamma=1.0, Z_0=0.06, amp=0.37, R_inner=R_MARS, R_outer=R_KUIPER_BELT)),
    L.INNER_NARROW_BAND: (
        NarrowBand,
        dict(_RRM_PLANE, A=0.04, gamma=1.0, beta_nb=9.35, G=0.12, R_inner=R_MARS, R_outer=R_ASTEROID_BELT),
    ),
    L.OUTER_NARROW_BAND: (
        NarrowBand,
        dict(_RRM_PLANE, A=0.032, gamma=1.0, beta_nb=1.42, G=0.6, R_inner=R_MARS, R_outer=R_ASTEROID_BELT),
    ),
    L.BROAD_BAND: (
        BroadBand,
        dict(x_0=0.0, y_0=0.0, z_0=0.0, i=2.6, Omega=110.0, A=0.051, gamma=1.0, beta_bb=9.3, sigma_bb=5.0,
             R_inner=R_MARS, R_outer=R_ASTEROID_BELT),
    ),
    L.INTERSTELLAR: (Interstellar, dict(x_0=0.0, y_0=0.0, z_0=0.0, i=0.0, Omega=0.0, amp=0.010)),
    L.RING_RRM: (
        RingRRM,
        dict(A=0.16, x_0=0.0, y_0=0.0, z_0=0.0, i=0.49, Omega=22.3, n_0=1.0, R=1.03, sigma_r=0.025, sigma_z=0.054),
    ),
    L.FEATURE_RRM: (
        FeatureRRM,
        dict(A=0.065, x_0=0.0, y_0=0.0, z_0=0.0, i=0.49, Omega=22.3, n_0=1.0, R=1.06, sigma_r=0.10, sigma_z=0.091,
             theta=-10.0, sigma_theta=12.1),
    ),
}
T_LARGE_GRAINS, T_SMALL_GRAINS = 255.0, 305.0
DELTA_LARGE_GRAINS, DELTA_SMALL_GRAINS = 0.5, 0.4
T_0_RRM = {lbl: (T_SMALL_GRAINS if lbl == L.INTERSTELLAR else T_LARGE_GRAINS) for lbl in RRM_COMPONENTS}
DELTA_RRM = {lbl: (DELTA_SMALL_GRAINS if lbl == L.INTERSTELLAR else DELTA_LARGE_GRAINS) for lbl in RRM_COMPONENTS}
CALIBRATION_RRM = [1.0, 1.0, 1.0, 1.0]
PLANCK_BANDS_GHZ = [100.0, 143.0, 217.0, 353.0, 545.0, 857.0]

_E_BAND_DIRBE = [
    1.0,
    1.0,
    1.659892404064974,
    0.3592645195835044,
    1.0127926948497732,
    1.0,
    1.2539242027824944,
    1.5167023376593836,
    1.1317240279481993,
    1.3996145963796358,
]
_E_RING_DIRBE = [
    1.0,
    1.0,
    1.659892404064974,
    1.0675116768340536,
    1.0608768682182081,
    1.0,
    0.8726636137878518,
    1.0985346556794289,
    1.1515825707787077,
    0.8576380099421744,
]
DIRBE_EMISSIVITY = {
    L.CLOUD: [
        1.0,
        1.0,
        1.659892404064974,
        0.9974090848665298,
        0.9576691480594887,
        1.0,
        0.7333883261676887,
        0.6478988180222407,
        0.6769420588104739,
        0.5191208540195074,
    ],
    L.BAND1: list(_E_BAND_DIRBE),
    L.BAND2: list(_E_BAND_DIRBE),
    L.BAND3: list(_E_BAND_DIRBE),
    L.RING: list(_E_RING_DIRBE),
    L.FEATURE: list(_E_RING_DIRBE),
}
_A_DIRBE = [0.20411939612669797, 0.255211328920523, 0.21043660481632315] + [0.0] * 7
DIRBE_ALBEDO = {label: list(_A_DIRBE) for label in DIRBE_COMPONENTS}
DIRBE_SOLAR_IRRADIANCE = [
    234056060.0,
    123098740.0,
    64292872.0,
    35733824.0,
    5763843.0,
    1327989.4,
    230553.73,
    82999.336,
    42346.605,
    14409.608,
]
DIRBE_C1 = [-0.94209999, -0.52670002, -0.4312] + [0.0] * 7
DIRBE_C2 = [0.1214, 0.18719999, 0.1715] + [0.0] * 7
DIRBE_C3 = [-0.1648, -0.59829998, -0.63330001] + [0.0] * 7

PLANCK13_EMISSIVITY = {
    L.CLOUD: [0.003, -0.014, 0.031, 0.168, 0.223, 0.301],
    L.BAND1: [1.129, 1.463, 2.024, 2.035, 2.235, 1.777],
    L.BAND2: [0.674, 0.53, 0.338, 0.436, 0.718, 0.716],
    L.BAND3: [1.106, 1.794, 2.507, 2.4, 3.193, 2.87],
    L.RING: [0.163, -0.252, -0.185, -0.211, 0.591, 0.578],
    L.FEATURE: [0.252, -0.002, 0.243, 0.676, -0.182, 0.423],
}
PLANCK15_EMISSIVITY = {
    L.CLOUD: [0.012, 0.022, 0.051, 0.106, 0.167, 0.256],
    L.BAND1: [1.02, 1.23, 1.3, 1.58, 1.74, 2.06],
    L.BAND2: [0.08, 0.15, 0.15, 0.39, 0.54, 0.85],
    L.BAND3: [0.72, 1.16, 1.27, 1.88, 2.54, 3.37],
}
PLANCK18_EMISSIVITY = {
    L.CLOUD: [0.018, 0.02, 0.042, 0.082, 0.179, 0.304],
    L.BAND1: [0.54, 1.0, 1.11, 1.52, 1.47, 1.58],
    L.BAND2: [0.07, 0.17, 0.21, 0.35, 0.49, 0.7],
    L.BAND3: [0.19, 0.84, 1.12, 1.77, 1.84, 2.11],
}
ODEGARD_EMISSIVITY = {
    L.CLOUD: [0.014, 0.023, 0.063, 0.132, 0.21, 0.285],
    L.BAND1: [1.25, 1.39, 1.85, 2.41, 2.81, 3.23],
    L.BAND2: [0.15, 0.22, 0.4, 0.8, 1.11, 1.58],
    L.BAND3: [0.5, 0.89, 1.22, 1.96, 2.81, 3.6],
}

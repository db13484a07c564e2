"""Face-state families for the per-face Riemann solver checks.

Each family is a seeded draw of (wl, wr, bx): primitive states in the solvers' local order
(density, normal and two transverse velocities, gas pressure, two transverse fields) and
the normal field.  Velocities are 3-velocities for the Newtonian solvers and spatial
4-velocities for the relativistic ones, so every draw is a valid state for both.  The
families reach every region of the relativistic HLLD fan (L, R, the HLL fallback, aL,
aR, the contact) and the solvers' degenerate cases (equal states, zero normal field,
pure hydrodynamics, near-vacuum, static field-only states).
"""
import numpy as np

FAMILIES = ("mild", "shock", "magnetised", "ultra", "zero_bx", "equal", "hydro",
            "near_vacuum", "static")


def _state(rng, n, rho, v, p, bt):
    return np.column_stack([rng.uniform(*rho, n), rng.normal(0, v, (n, 3)),
                            rng.uniform(*p, n), rng.normal(0, bt, (n, 2))])


def faces(family, n, seed=0):
    rng = np.random.default_rng([seed, FAMILIES.index(family)])
    if family == "mild":            # smooth flow: small jumps
        wl = _state(rng, n, (.5, 2), .3, (.1, 2), .5)
        wr = wl * (1 + rng.normal(0, .05, wl.shape))
        bx = rng.normal(0, .5, n)
    elif family == "shock":         # independent L and R states: strong jumps
        wl = _state(rng, n, (.1, 10), 3, (.01, 100), 3)
        wr = _state(rng, n, (.1, 10), 3, (.01, 100), 3)
        bx = rng.normal(0, 3, n)
    elif family == "magnetised":    # magnetic pressure far above gas pressure
        wl = _state(rng, n, (.01, 1), 1, (1e-3, .1), 10)
        wr = _state(rng, n, (.01, 1), 1, (1e-3, .1), 10)
        bx = rng.normal(0, 10, n)
    elif family == "ultra":         # Lorentz factors of tens
        wl = _state(rng, n, (.1, 1), 30, (.01, 1), 1)
        wr = _state(rng, n, (.1, 1), 30, (.01, 1), 1)
        bx = rng.normal(0, 1, n)
    elif family == "zero_bx":
        wl = _state(rng, n, (.5, 2), .5, (.1, 2), .5)
        wr = _state(rng, n, (.5, 2), .5, (.1, 2), .5)
        bx = np.zeros(n)
    elif family == "equal":         # no jump at all
        wl = _state(rng, n, (.5, 2), .3, (.1, 2), .5)
        wr = wl.copy()
        bx = rng.normal(0, .5, n)
    elif family == "hydro":         # no field
        wl = _state(rng, n, (.5, 2), .3, (.1, 2), .5)
        wl[:, 5:] = 0.0
        wr = wl * (1 + rng.normal(0, .1, wl.shape))
        bx = np.zeros(n)
    elif family == "near_vacuum":   # one side nearly empty
        wr = _state(rng, n, (.5, 2), .3, (.1, 2), .5)
        wl = wr.copy()
        wl[:, 0] = 1e-12
        wl[:, 4] = 1e-14
        bx = rng.normal(0, .5, n)
    else:                           # "static": at rest, normal field only
        wl = _state(rng, n, (.5, 2), .3, (.1, 2), .5)
        wl[:, 1:4] = 0.0
        wl[:, 5:] = 0.0
        wr = wl.copy()
        bx = rng.normal(0, .5, n)
    return wl, wr, bx


def face_velocity_differences(wl, wr, seed=0):
    """(dvn, dvt) per face for the low-dissipation HLLD: the normal-velocity jump of the
    two states and a seeded transverse difference, both sides of zero (compression and
    expansion; the shock detector saturates for dvt >= dvn)."""
    rng = np.random.default_rng([seed, 99])
    dvn = wr[:, 1] - wl[:, 1]
    dvt = rng.normal(0.0, 0.5, wl.shape[0]) * (1.0 + np.abs(dvn))
    return np.column_stack([dvn, dvt])

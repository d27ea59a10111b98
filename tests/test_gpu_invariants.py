"""Size-independent properties of the device loops at the benchmark sizes,
where the CPU oracle would take minutes: on a periodic box with exactly
uniform metrics, translating the initial state by whole cells translates the
solution, bit for bit, in the exact policy (the tiles, z chunks and block
boundaries of the kernels must not show).  The shifts are not multiples of
any tile edge."""
import numpy as np
import pytest

import oracle
from utrip_gb300 import drivers, setups

pytestmark = pytest.mark.gpu


def uniform(s, axes):
    out = dict(s)
    for a in axes:
        for k in ("d" + a, "d" + a + "m"):
            out[k] = np.full(np.asarray(s[k]).size, float(np.asarray(s[k])[1]))
    return out


def shifted(s, shift):
    m = s["margin"]
    inner = tuple(slice(m, -m) for _ in shift)
    st = []
    for a in setups.copy_state(s):
        b = a.copy(order="F")
        b[inner] = np.roll(a[inner], shift, axis=tuple(range(len(shift))))
        st.append(b)
    apply = oracle.apply_bc_program_3d if len(shift) == 3 else oracle.apply_bc_program
    apply(st, s["bc"], m, s)
    return st


def check(s, shift, nsteps):
    # both runs start from ghost cells filled by the periodic rule (a set-up
    # may evaluate its ghost cells analytically, a last-bit difference)
    base = shifted(s, (0,) * len(shift))
    moved = shifted(s, shift)
    out1 = drivers.run_resident(s, base, nsteps, exact=True)
    out2 = drivers.run_resident(s, moved, nsteps, exact=True)
    assert out1 == out2  # same dt sequence: the CFL minimum ignores order
    m = s["margin"]
    inner = tuple(slice(m, -m) for _ in shift)
    for k, a, b in zip(s["names"], base, moved):
        want = np.roll(a[inner], shift, axis=tuple(range(len(shift))))
        assert np.array_equal(b[inner], want), k


@pytest.mark.parametrize("solver,n,margin", [("mlw_m3", 512, 1), ("roe_m3", 256, 3)])
def test_translation_2d_exact(gpu, solver, n, margin):
    """Roe runs with margin 3: with 2, cells next to the ghost layer read the
    outer layer's half-step values, which roe_m3 never updates (the input
    primitives stand there), so translation moves them."""
    s = uniform(setups.orszag_tang(n, solver=solver, margin=margin), "xy")
    check(s, (37, 101), 20)


@pytest.mark.parametrize("solver", ["mlw_m_3d", "roe_m_3d", "hlld_3d"])
def test_translation_3d_exact(gpu, solver):
    s = uniform(setups.turbulence_3d(64 if solver != "mlw_m_3d" else 128, solver=solver),
                "xyz")
    check(s, (5, 17, 33), 8)

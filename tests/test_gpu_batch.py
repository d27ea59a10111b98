"""GPU tests of the batched 2-D runs (cans_batch_*): every run of a batch of
uneven grid sizes and plasma betas ends bit-identical to the same run done
alone (and, in the exact policy, to the CPU oracle), for every tile
configuration the autotuner can pick."""
import numpy as np
import pytest

import oracle
from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu


def _sweep(sizes, betas, seed=4):
    return [setups.shear_layer(n, beta=b, ny=m, seed=seed + k)
            for k, ((n, m), b) in enumerate(zip(sizes, betas))]


def _assert_same(names, got, ref, what):
    for k, a, b in zip(names, got, ref):
        if not np.array_equal(a, b):
            raise AssertionError(f"{what} {k}: {int(np.sum(a != b))} cells differ, "
                                 f"max {float(np.max(np.abs(a - b))):.3e}")


@pytest.mark.parametrize("exact", [True, False])
def test_batch_equals_single_runs(gpu, exact):
    runs = _sweep([(40, 36), (66, 48), (33, 70), (80, 80), (47, 29)],
                  [0.1, 0.5, 1.0, 3.0, 10.0])
    b = capi.Batch(runs, exact=exact)
    try:
        for g, s in enumerate(runs):
            b.push(g, s["state"])
        b.start(nstop=25, safety=0.4, dtmin=1e-10)
        b.advance(30)  # the loop of every run ends at ns = 25
        for g, s in enumerate(runs):
            st = b.query(g)
            assert st.done and st.ns == 25 and st.nexec == 25 and st.merr == 0
            got = b.pull(g)
            ref = setups.copy_state(s)
            t, ns, merr, nexec = drivers.run_resident(s, ref, 25, exact=exact)
            assert (ns, nexec) == (25, 25)
            if exact:
                assert st.t == t
                _assert_same(s["names"], got, ref, f"grid {g}")
            else:
                # the fast policy leaves FMA contraction to the compiler, which
                # may contract the batched and the single-run kernels apart
                assert abs(st.t - t) <= 1e-13 * t
                for k, a, r in zip(s["names"], got, ref):
                    scale = max(float(np.max(np.abs(r))), 1e-300)
                    assert float(np.max(np.abs(a - r))) <= 1e-12 * scale, (g, k)
    finally:
        b.close()


def test_batch_matches_oracle_exact(gpu, oracle_lib):
    runs = _sweep([(34, 30), (52, 40)], [0.3, 2.0])
    b = capi.Batch(runs, exact=True)
    try:
        for g, s in enumerate(runs):
            b.push(g, s["state"])
        b.start(nstop=15, safety=0.4, dtmin=1e-10)
        b.advance(15)
        for g, s in enumerate(runs):
            ref = setups.copy_state(s)
            t_ref, ns_ref, _, _ = oracle.run_2d(s, ref, 15)
            assert b.query(g).t == t_ref
            _assert_same(s["names"], b.pull(g), ref, f"grid {g}")
    finally:
        b.close()


def test_every_config_agrees_and_autotune_keeps_state(gpu):
    runs = _sweep([(70, 44), (38, 90), (129, 65)], [0.2, 1.0, 5.0])
    results = []
    for cfg in range(capi.batch_configs()):
        b = capi.Batch(runs, exact=True)
        try:
            for g, s in enumerate(runs):
                b.push(g, s["state"])
            b.set_config(cfg)
            b.start(nstop=8, safety=0.4, dtmin=1e-10)
            b.advance(8, use_graph=(cfg % 2 == 0))
            results.append([b.pull(g) for g in range(len(runs))])
        finally:
            b.close()
    for cfg in range(1, len(results)):
        for g, s in enumerate(runs):
            _assert_same(s["names"], results[cfg][g], results[0][g], f"config {cfg} grid {g}")
    b = capi.Batch(runs, exact=True)
    try:
        for g, s in enumerate(runs):
            b.push(g, s["state"])
        b.start(nstop=8, safety=0.4, dtmin=1e-10)
        before = [b.pull(g) for g in range(len(runs))]
        cfg = b.autotune(2)
        assert 0 <= cfg < capi.batch_configs()
        for g, s in enumerate(runs):
            _assert_same(s["names"], b.pull(g), before[g], f"autotune grid {g}")
        b.advance(8)
        for g, s in enumerate(runs):
            _assert_same(s["names"], b.pull(g), results[0][g], f"after autotune grid {g}")
    finally:
        b.close()

"""Autotuner and its knobs: every candidate-cache buffer and every BP launch
variant gives the same edges and (to rounding) the same energies and forces;
the autotuner restores the state it tuned from."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAPHS = ["rotamer", "hbond_coverage", "protein_hbond", "environment_coverage_sc"]


def _batch(syn_configs):
    import upside_gb300 as U
    (p60, z60), (p150, z150) = syn_configs[60], syn_configs[150]
    b = U.Batch([p60, p150, p150])
    b.set_pos(np.concatenate([z60["pos"][0], z150["pos"][0], z150["pos"][1]]))
    b.set_thermostat([0.85, 0.9, 0.95], np.array([1, 2, 3], np.uint32))
    return b


def test_tuning_knobs_do_not_change_results(syn_configs):
    b = _batch(syn_configs)
    b.run(10, use_graph=True, graph_rounds=5)
    x = b.get_pos()
    e0, f0 = b.evaluate()
    edges0 = {g: b.node_edges(g) for g in GRAPHS}
    for scale in (1.0, 2.0, 3.0):
        for variant in range(9):
            b.set_tuning(scale, variant, (1, 2, 4, 8)[variant % 4])
            b.set_pos(x)
            e, f = b.evaluate()
            for g in GRAPHS:
                assert np.array_equal(b.node_edges(g), edges0[g]), (scale, variant, g)
            assert np.abs(e - e0).max() <= 1e-5 * max(1.0, np.abs(e0).max()), (scale, variant)
            assert np.abs(f - f0).max() <= 1e-4 * np.abs(f0).max(), (scale, variant)


def test_autotune_restores_state_and_reports(syn_configs):
    b = _batch(syn_configs)
    b.run(10, use_graph=True, graph_rounds=5)
    x, m = b.get_pos(), b.get_mom()
    trials, chosen = b.autotune(2)
    # 5 buffer scales, 9 BP variants, 5 stream counts, and when the two
    # fastest BP variants are within 8%, both timed again
    finals = [k for k in trials if k.startswith("final_bp_variant_")]
    assert len(trials) == 5 + 9 + 5 + len(finals) and len(finals) in (0, 2) and chosen
    assert all(v > 0 for v in trials.values())
    assert np.array_equal(b.get_pos(), x) and np.array_equal(b.get_mom(), m)
    b.run(2, use_graph=True, graph_rounds=1)
    assert b.status() & 3 == 0

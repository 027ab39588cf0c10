"""Launch configuration and the autotuner: every configuration gives bit-identical results, and
the autotuner's tuning steps are ordinary steps of the world."""
import numpy as np
import pytest

import b2g
import parity
import scenes

pytestmark = pytest.mark.gpu


def _world(scene):
    w = b2g.B2world(gravity=scene["gravity"], num_worlds=scene.get("num_worlds", 1))
    w.set_allow_sleeping(False)
    w.set_continuous_physics(False)
    scenes.build_world(w, scene)
    return w


@pytest.mark.parametrize("cfg", [dict(coop_blocks_per_sm=2, collide_block=64, traverse_block=64, solver_block=256,
                                      collide_group=8),
                                 dict(coop_blocks_per_sm=1, collide_block=256, traverse_block=32, solver_block=512,
                                      collide_group=32)])
def test_configurations_give_identical_results(built, cfg):
    s = scenes.mixed(n_circles=300, n_polygons=300, size=25.0, seed=21)
    a, b = _world(s), _world(s)
    b.set_launch_config(**cfg)
    assert b.get_launch_config() == cfg
    for _ in range(120):
        a.step(s["dt"], s["vi"], s["pi"])
        b.step(s["dt"], s["vi"], s["pi"])
    sa, sb = a.get_body_states(), b.get_body_states()
    for f in parity.BODY_FIELDS:
        assert np.array_equal(sa[f], sb[f]), f
    a.close()
    b.close()


def test_autotune_steps_are_ordinary_steps(built):
    s = scenes.batched(num_worlds=16, lo=16, hi=256, seed=3)
    a, b = _world(s), _world(s)
    per = 2
    cfg = b.autotune(s["dt"], s["vi"], s["pi"], per)
    assert cfg["coop_blocks_per_sm"] in (1, 2)
    assert cfg["collide_block"] in (64, 128, 256) and cfg["traverse_block"] in (64, 128, 256)
    assert cfg["solver_block"] in (256, 512)
    assert cfg["collide_group"] in (0, 8, 32)
    n = b.tuning_steps()
    assert n >= 2 * 3 * 3  # at least the two block-size knobs, every candidate stepped 2 + 1 times
    for _ in range(n):
        a.step(s["dt"], s["vi"], s["pi"])
    sa, sb = a.get_body_states(), b.get_body_states()
    for f in parity.BODY_FIELDS:
        assert np.array_equal(sa[f], sb[f]), f
    # a later world of the same size bucket starts with the tuned configuration
    c = _world(s)
    c.step(s["dt"], s["vi"], s["pi"])  # the configuration is applied when the world is first uploaded
    assert c.get_launch_config() == cfg
    for w in (a, b, c):
        w.close()


def test_invalid_configuration_is_rejected(built):
    s = scenes.pyramid(rows=3)
    w = _world(s)
    with pytest.raises(b2g.B2GError):
        w.set_launch_config(coop_blocks_per_sm=3)
    with pytest.raises(b2g.B2GError):
        w.set_launch_config(collide_block=100)
    with pytest.raises(b2g.B2GError):
        w.set_launch_config(solver_block=384)
    with pytest.raises(b2g.B2GError):
        w.set_launch_config(collide_group=33)
    w.close()

"""CPU: the uneven-batch autotuner's host logic -- candidate names, the
candidate list per set of geometries, strategy validation (no GPU calls)."""
from types import SimpleNamespace

import pytest

from vmbd_gb300 import autotune


def fake_plan(sw, sf, N):
    # the attributes the candidate logic reads
    return SimpleNamespace(winaux=SimpleNamespace(sw=sw), sf=sf, N=N)


def test_parse_candidate_names():
    assert autotune.parse("persistent") == ("persistent", 0, 0)
    assert autotune.parse("per_class/cta") == ("per_class/cta", 0, 0)
    assert autotune.parse("per_class/cta@f192") == ("per_class/cta", 192, 0)
    assert autotune.parse("per_class/cluster@f192/t256") == ("per_class/cluster", 192, 256)
    assert autotune.parse("per_class/cta@t384") == ("per_class/cta", 0, 384)
    for bad in ("persistent@x192", "per_class/cta@f", "per_class/cta@f192/q1"):
        with pytest.raises(ValueError):
            autotune.parse(bad)


def test_candidates_add_frame_192_only_where_it_fits():
    # extent 118 (frame 128): power-of-two strategies only
    small = fake_plan((108, 108), (11, 11), 128)
    assert autotune.candidates([small]) == autotune.STRATEGIES
    # extent 144 on frame 256: the 192-frame variants, 256-thread CTAs per class only
    mid = fake_plan((120, 120), (25, 25), 256)
    c = autotune.candidates([small, mid])
    assert c[:3] == autotune.STRATEGIES
    assert {s + "@f192" for s in autotune.STRATEGIES} <= set(c)
    assert "per_class/cta@f192/t256" in c and "per_class/cluster@f192/t256" in c
    assert "persistent@f192/t256" not in c
    # already on 192, or too large for it: nothing to add
    assert autotune.candidates([fake_plan((120, 120), (25, 25), 192)]) == autotune.STRATEGIES
    assert autotune.candidates([fake_plan((164, 164), (31, 31), 256)]) == autotune.STRATEGIES


def test_variant_plans_keep_plans_without_options():
    plans = [fake_plan((108, 108), (11, 11), 128), fake_plan((120, 120), (25, 25), 256)]
    assert autotune.variant_plans(plans) == plans
    # a frame not smaller than the class's own: unchanged
    assert autotune.variant_plans(plans[:1], frame=192) == plans[:1]


def test_batch_runner_rejects_unknown_strategy():
    with pytest.raises(ValueError):
        autotune.BatchRunner([fake_plan((108, 108), (11, 11), 128)], [1], "per_image")

"""PlanConfig validation (host only)."""
import pytest

from stile_gb300.api import PlanConfig


@pytest.mark.parametrize("path", ["hybrid", "csr", "auto"])
def test_paths_accepted(path):
    assert PlanConfig(path=path).path == path


@pytest.mark.parametrize("kw", [dict(path="dense"), dict(path=""), dict(backward="both"), dict(backward=None)])
def test_unknown_path_or_backward_rejected(kw):
    with pytest.raises(ValueError):
        PlanConfig(**kw)


def test_path_and_backward_do_not_change_the_plan_key():
    """The plan cache keys on the search settings only: the same plan serves
    every path and backward variant."""
    assert PlanConfig(path="auto", backward="fused").search_kwargs().keys() == PlanConfig().search_kwargs().keys()
    assert "path" not in PlanConfig().search_kwargs() and "backward" not in PlanConfig().search_kwargs()

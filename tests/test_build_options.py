"""Build-time options of gpusnarks_gb300/build.py (no compilation here)."""
import pytest

from gpusnarks_gb300 import build as B


def test_schedule_option_becomes_a_define(monkeypatch):
    monkeypatch.delenv("GSN_MONT_SCHEDULE", raising=False)
    assert B._defines() == []
    monkeypatch.setenv("GSN_MONT_SCHEDULE", "2")
    assert B._defines() == ["-DGSN_MONT_SCHEDULE=2"]


def test_schedule_option_must_be_a_number(monkeypatch):
    monkeypatch.setenv("GSN_MONT_SCHEDULE", "2; rm -rf /")
    with pytest.raises(ValueError):
        B._defines()

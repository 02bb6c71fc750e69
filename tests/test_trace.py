"""NVTX stages (harmonica_gb300._trace): balanced push/pop, exceptions
propagate, and the ranges can be switched off or be absent without any
effect on the traced code."""

import pytest

from harmonica_gb300 import _trace


class _Recorder:
    def __init__(self):
        self.calls = []

    def range_push(self, name):
        self.calls.append(("push", name))

    def range_pop(self):
        self.calls.append(("pop",))


def test_stage_pushes_and_pops(monkeypatch):
    rec = _Recorder()
    monkeypatch.setattr(_trace, "_nvtx", rec)
    with _trace.stage("forward"):
        with _trace.stage("download"):
            pass
    assert rec.calls == [("push", "hg:forward"), ("push", "hg:download"), ("pop",), ("pop",)]


def test_stage_pops_when_the_traced_code_raises(monkeypatch):
    rec = _Recorder()
    monkeypatch.setattr(_trace, "_nvtx", rec)
    with pytest.raises(ValueError, match="boom"):
        with _trace.stage("checks"):
            raise ValueError("boom")
    assert rec.calls == [("push", "hg:checks"), ("pop",)]


def test_switched_off_by_environment(monkeypatch):
    monkeypatch.setattr(_trace, "_nvtx", None)
    monkeypatch.setenv("HG_NVTX", "0")
    assert not _trace.enabled()
    with _trace.stage("forward"):
        value = 1
    assert value == 1


def test_without_nvtx_support(monkeypatch):
    """A torch build whose NVTX calls fail traces nothing and breaks nothing."""
    import torch

    def unavailable(*args, **kwargs):
        raise RuntimeError("NVTX functions not installed")

    monkeypatch.setattr(_trace, "_nvtx", None)
    monkeypatch.delenv("HG_NVTX", raising=False)
    monkeypatch.setattr(torch.cuda.nvtx, "range_push", unavailable)
    assert not _trace.enabled()
    with _trace.stage("forward"):
        value = 2
    assert value == 2

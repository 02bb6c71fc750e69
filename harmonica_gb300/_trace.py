"""
NVTX ranges around the host stages of the forward calls (checks, uploads,
kernel launches, downloads), so that a profiler's timeline (Nsight Systems,
or ``ncu --nvtx`` filters) shows where a call spends its time.

Ranges are named ``hg:<stage>``.  They are on by default and cost about a
microsecond each; ``HG_NVTX=0`` turns them off.  Tracing never affects a
result: where the torch build has no NVTX support the ranges are empty
context managers.
"""

import contextlib
import os

_nvtx = None  # torch.cuda.nvtx once probed and usable, False when unusable


def _probe():
    global _nvtx
    if os.environ.get("HG_NVTX", "1") == "0":
        _nvtx = False
        return _nvtx
    try:
        import torch  # noqa: PLC0415

        torch.cuda.nvtx.range_push("hg:probe")
        torch.cuda.nvtx.range_pop()
        _nvtx = torch.cuda.nvtx
    except Exception:  # noqa: BLE001 - no NVTX in this torch build: trace nothing
        _nvtx = False
    return _nvtx


@contextlib.contextmanager
def stage(name):
    """An NVTX range ``hg:<name>`` around the enclosed host code."""
    nvtx = _nvtx if _nvtx is not None else _probe()
    if not nvtx:
        yield
        return
    nvtx.range_push("hg:" + name)
    try:
        yield
    finally:
        nvtx.range_pop()


def enabled():
    """Whether stages are recorded as NVTX ranges in this process."""
    return bool(_nvtx if _nvtx is not None else _probe())

"""Optional per-stage CUDA-event timing of the Meshoid pipeline.

    rec = StageRecorder(); set_recorder(rec)
    ...            # Meshoid / D calls record events on the current stream
    torch.cuda.synchronize(); rec.totals()   # {stage: milliseconds}

With no recorder installed (the default) the hooks cost one None check.
"""
from __future__ import annotations

import contextlib

import torch

_recorder = None


def set_recorder(rec):
    global _recorder
    _recorder = rec


class StageRecorder:
    def __init__(self):
        self.events = []  # (name, start, end)

    def reset(self):
        self.events.clear()

    def totals(self):
        out = {}
        for name, a, b in self.events:
            out[name] = out.get(name, 0.0) + a.elapsed_time(b)
        return out

    def counts(self):
        out = {}
        for name, _, _ in self.events:
            out[name] = out.get(name, 0) + 1
        return out


@contextlib.contextmanager
def stage(name: str):
    rec = _recorder
    if rec is None:
        yield
        return
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    try:
        yield
    finally:
        b.record()
        rec.events.append((name, a, b))


"""bench.timed_frames on the CPU with a fake solver and fake CUDA events.

Every timed frame must find the previous frame finished (its status read back) and the L2
flush queued before its start event, so that the frame graph is queued while the device
writes the flush and the host's turnaround stays outside the frame's events; per_frame adds
each frame's event time and kernel count."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


class _Event:
    log = None

    def __init__(self, enable_timing=False):
        self.t = None

    def record(self, stream=None):
        _Event.log.append("event")
        self.t = float(len(_Event.log))

    def elapsed_time(self, end):
        return end.t - self.t


class _Solver:
    def __init__(self, log, kernels_per_frame=(340, 330)):
        self.log = log
        self.kernels = 0
        self.frame = 0
        self.per_frame = kernels_per_frame

    @property
    def kernels_launched(self):
        return self.kernels

    def sync(self):
        self.log.append("sync")

    def step_async(self, dt, substeps, iterations):
        self.log.append("launch")
        self.kernels += self.per_frame[self.frame % len(self.per_frame)]
        self.frame += 1


@pytest.fixture
def bench_fakes(monkeypatch):
    import torch

    import bench

    log = []
    _Event.log = log
    monkeypatch.setattr(torch.cuda, "Event", _Event)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: log.append("device sync"))
    return bench, log


def test_previous_frame_and_flush_come_before_the_start_event(bench_fakes):
    bench, log = bench_fakes
    total = bench.timed_frames(_Solver(log), None, 3, lambda: log.append("flush"))
    frame = ["sync", "flush", "event", "launch", "event"]
    assert log == frame * 3 + ["sync", "device sync"]
    assert total == pytest.approx(3 * 2.0)  # each frame's events bracket only its launch


def test_without_flush_the_frame_still_waits_outside_its_events(bench_fakes):
    bench, log = bench_fakes
    bench.timed_frames(_Solver(log), None, 2)
    assert log == ["sync", "event", "launch", "event"] * 2 + ["sync", "device sync"]


def test_per_frame_times_and_kernel_counts(bench_fakes):
    bench, log = bench_fakes
    total, times, kernels = bench.timed_frames(_Solver(log), None, 4, lambda: log.append("flush"), per_frame=True)
    assert len(times) == 4 and total == pytest.approx(sum(times))
    assert kernels == [340, 330, 340, 330]

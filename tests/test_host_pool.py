"""The page-locked output pool of MPMSolver._to_host (particle_info): a
buffer is handed out again only when no caller holds its array or a view of
it, and eviction never drops a held buffer.  Run on the CPU with ordinary
tensors standing in for page-locked ones."""
import torch

import taichi_elements_gb300.mpm_solver as M


def _fake_pool(monkeypatch, cap):
    made = []
    real_empty = torch.empty

    def empty(shape, dtype=None, pin_memory=False):
        made.append(tuple(shape))
        return real_empty(shape, dtype=dtype)

    monkeypatch.setattr(M.torch, "empty", empty)
    monkeypatch.setattr(M, "_pinned_pool", [])
    monkeypatch.setattr(M, "_PINNED_POOL_BYTES", cap)
    return made


def test_held_buffers_are_not_reused(monkeypatch):
    made = _fake_pool(monkeypatch, 1 << 30)
    _, a = M._pinned_buffer((8, 3), torch.float32)
    _, b = M._pinned_buffer((8, 3), torch.float32)
    assert a is not b and len(made) == 2
    view = b[:, 0]
    del b
    _, c = M._pinned_buffer((8, 3), torch.float32)  # a held, b held through a view
    assert len(made) == 3 and c is not a
    del a
    _, d = M._pinned_buffer((8, 3), torch.float32)  # a released: its buffer returns
    assert len(made) == 3 and view.base is not d


def test_eviction_keeps_held_buffers(monkeypatch):
    _fake_pool(monkeypatch, 100)
    _, a = M._pinned_buffer((40,), torch.float32)
    _, b = M._pinned_buffer((40,), torch.float32)
    del b
    _, c = M._pinned_buffer((41,), torch.float32)
    shapes = [tuple(q[0].shape) for q in M._pinned_pool]
    assert shapes == [(40,), (41,)] and M._pinned_pool[0][1] is a

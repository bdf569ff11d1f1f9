"""Helpers for the GPU tests: move raw-bit numpy arrays to/from the device
(torch byte tensors) and run a sort through the C ABI."""

from __future__ import annotations

import numpy as np


def to_dev(torch, arr: np.ndarray):
    a = np.ascontiguousarray(arr)
    return torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).cuda()


def from_dev(t, like: np.ndarray) -> np.ndarray:
    return t.cpu().numpy().view(like.dtype).reshape(like.shape)


def value_bytes_of(vals) -> int:
    if vals is None:
        return 0
    return vals.dtype.itemsize * (vals.shape[1] if vals.ndim == 2 else 1)


def gpu_sort(gb, torch, kt: str, raw: np.ndarray, desc: bool = False, vals: np.ndarray | None = None,
             stream=None, garbage_workspace: bool = False, key_offset: int = 0, val_offset: int = 0):
    """Sorts copies of raw (and vals) on the device; returns host arrays.
    key_offset / val_offset shift the device pointers by that many elements
    (unaligned-pointer cases)."""
    n = raw.shape[0]
    vb = value_bytes_of(vals)
    kb = raw.dtype.itemsize * (raw.shape[1] if raw.ndim == 2 else 1)
    dk = torch.zeros(max(1, (n + key_offset) * kb), dtype=torch.uint8, device="cuda")
    if n:
        dk[key_offset * kb:(key_offset + n) * kb] = to_dev(torch, raw)
    dv = None
    if vals is not None:
        dv = torch.zeros(max(1, (n + val_offset) * vb), dtype=torch.uint8, device="cuda")
        if n:
            dv[val_offset * vb:(val_offset + n) * vb] = to_dev(torch, vals)
    tb = gb.temp_bytes(kt, n, vb)
    ws = torch.empty(max(tb, 1), dtype=torch.uint8, device="cuda")
    if garbage_workspace:
        ws.random_(0, 256)
    kptr = dk.data_ptr() + key_offset * kb
    vptr = None if dv is None else dv.data_ptr() + val_offset * vb
    gb.sort(kptr, n, kt, ws, tb, values=vptr, value_bytes=vb, descending=desc, stream=stream)
    torch.cuda.synchronize()
    st = gb.workspace_status(kt, n, ws, vb)
    assert st == gb.OK, gb.status_string(st)
    k = from_dev(dk[key_offset * kb:(key_offset + n) * kb], raw) if n else raw.copy()
    if vals is None:
        return k
    v = from_dev(dv[val_offset * vb:(val_offset + n) * vb], vals) if n else vals.copy()
    return k, v

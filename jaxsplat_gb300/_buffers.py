"""Named fp32 views of one device (or pinned host) buffer."""

from __future__ import annotations

import math

import torch


def block(shapes, device, pin=False):
    """One fp32 buffer holding the named shapes back to back, each starting on
    a 256-byte boundary; returns (buffer, {name: view})."""
    offs, total = [], 0
    for _, shape in shapes:
        offs.append(total)
        total += (math.prod(shape) + 63) // 64 * 64
    buf = torch.zeros(total, dtype=torch.float32, device=device, pin_memory=pin)
    return buf, {name: buf[o:o + math.prod(shape)].view(shape)
                 for (name, shape), o in zip(shapes, offs)}

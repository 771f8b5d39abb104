"""GPU power sampling around a region (rmq_power_begin / rmq_power_end).

The role of the reference's GPUPowerBegin / GPUPowerEnd
(common/nvmlPower.cpp): NVML board power read every ``sample_ms`` by a
native thread, integrated to energy, optionally written to the reference's
whitespace table.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

from ._native import load

__all__ = ["PowerSampler"]


class PowerSampler:
    """``with PowerSampler(device) as p: ...`` then ``p.avg_watts``,
    ``p.energy_joules``, ``p.seconds``; ``p.available`` is False (and the
    numbers None) when NVML cannot be used."""

    def __init__(self, device: int = 0, sample_ms: int = 100, cooldown_ms: int = 0,
                 path: Optional[str] = None):
        self.device, self.sample_ms, self.cooldown_ms, self.path = device, sample_ms, cooldown_ms, path
        self.available = False
        self.status = None
        self.avg_watts = self.energy_joules = self.seconds = None

    def __enter__(self):
        self.status = load().rmq_power_begin(self.device, self.sample_ms, self.cooldown_ms,
                                             self.path.encode() if self.path else None)
        self.available = self.status == 0
        return self

    def __exit__(self, *exc):
        if self.available:
            w, e, s = C.c_double(), C.c_double(), C.c_double()
            if load().rmq_power_end(self.cooldown_ms, C.byref(w), C.byref(e), C.byref(s)) == 0:
                self.avg_watts, self.energy_joules, self.seconds = w.value, e.value, s.value
        return False

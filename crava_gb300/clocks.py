"""Sample one GPU's SM clock and clock-event reasons through NVML, read-only.

    python -m crava_gb300.clocks --uuid GPU-xxxxxxxx-... --interval-ms 10

Prints one CSV line per sample, ``sm_mhz,max_sm_mhz,power_w,reasons`` (reasons
= NVML clock-event bit mask), until killed.  It runs as its own process so
that sampling takes no interpreter time from the process being measured; the
GPU is looked up by UUID because NVML numbers every GPU of the machine while
CUDA numbers only the visible ones.  Nothing here changes a GPU setting.
"""
from __future__ import annotations

import argparse
import ctypes as ct
import sys
import time

# NVML clock-event reason bits (nvmlClocksEventReason*)
REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
           0x80: "hw_power_brake_slowdown"}
NVML_CLOCK_SM = 1


def open_device(uuid):
    nv = ct.CDLL("libnvidia-ml.so.1")
    if nv.nvmlInit_v2() != 0:
        raise OSError("nvmlInit failed")
    h = ct.c_void_p()
    if nv.nvmlDeviceGetHandleByUUID(uuid.encode(), ct.byref(h)) != 0:
        raise OSError(f"no NVML device with UUID {uuid}")
    return nv, h


def sample(nv, h):
    sm, mx, mw, r = ct.c_uint(), ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
    nv.nvmlDeviceGetClockInfo(h, NVML_CLOCK_SM, ct.byref(sm))
    nv.nvmlDeviceGetMaxClockInfo(h, NVML_CLOCK_SM, ct.byref(mx))
    nv.nvmlDeviceGetPowerUsage(h, ct.byref(mw))
    fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or nv.nvmlDeviceGetCurrentClocksThrottleReasons
    fn(h, ct.byref(r))
    return sm.value, mx.value, mw.value / 1000.0, r.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--uuid", required=True)
    ap.add_argument("--interval-ms", type=float, default=10.0)
    a = ap.parse_args()
    nv, h = open_device(a.uuid)
    print("ready", flush=True)
    dt = a.interval_ms / 1e3
    while True:
        s = sample(nv, h)
        sys.stdout.write(f"{s[0]},{s[1]},{s[2]:.1f},{s[3]}\n")
        sys.stdout.flush()
        time.sleep(dt)


if __name__ == "__main__":
    main()

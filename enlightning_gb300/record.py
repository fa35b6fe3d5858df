"""Microphone files in the reference's format (enlightning.C:2392-2506).

The reference appends, after every step, one line per (level, patch)
containing a microphone to ``enlightning.record/mic-N.txt``:

    "%d %d %e\\n"  iteration, level, pressure            (enlightning.C:2471)

and, while the iteration is below the first source-pulse time, a baseline
line to ``mic-N-info.txt`` (preceded on iteration 1 by the microphone
number, the WAV sample rate and "(x,y)"):

    "%d %d %e %e\\n"  iteration, level, p0, sampled pressure   (:2455-2457)

``enlightning.record/mic.c`` (readMicFile, readInfoFile) reads both.  The
records come from the device (``Engine.mic_records``), already in the
reference's order: iteration, then microphone, level and patch.
"""
from __future__ import annotations

import os

import numpy as np


def c_e(v: float) -> str:
    """printf("%e") for a double (NaN and infinities spelled as glibc does)."""
    if np.isnan(v):
        return "-nan" if np.signbit(v) else "nan"
    if np.isinf(v):
        return "-inf" if v < 0 else "inf"
    return "%e" % v


def write_mic_files(records, directory, mic_positions, p0, wav_sample_rate, first_pulse_time=None):
    """Append the records to mic-N.txt / mic-N-info.txt under `directory`."""
    os.makedirs(directory, exist_ok=True)
    by_mic = {}
    for r in records:
        by_mic.setdefault(int(r["mic"]), []).append(r)
    for k, rows in sorted(by_mic.items()):
        n = k + 1
        with open(os.path.join(directory, f"mic-{n}.txt"), "a") as f:
            for r in rows:
                f.write(f"{int(r['iteration'])} {int(r['level'])} {c_e(float(r['p']))}\n")
        if first_pulse_time is None:
            continue
        info = [r for r in rows if int(r["iteration"]) < first_pulse_time]
        if not info:
            continue
        with open(os.path.join(directory, f"mic-{n}-info.txt"), "a") as f:
            x, y = mic_positions[k]
            for r in info:
                if int(r["iteration"]) == 1:  # written with every record of iteration 1, as the reference does
                    f.write(f"{n}\n{int(wav_sample_rate)}\n({'%g' % x},{'%g' % y})\n")
                f.write(f"{int(r['iteration'])} {int(r['level'])} {c_e(float(p0))} {c_e(float(r['p']))}\n")

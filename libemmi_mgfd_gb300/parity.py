"""Receiver-data comparison: how far one set of receiver data is from
another, in the terms the hot path is judged by -- amplitude error relative
to each channel's scale and phase error in degrees.

A channel's scale is its largest amplitude, but at least `floor` times the
largest amplitude of any channel of the same kind (E or H): channels that
vanish by symmetry hold only roundoff, which has no meaningful relative
error.  Phase is compared where the amplitude exceeds `floor` times the
scale.  The receiver data are the reference's dcal_fd layout per RHS,
[channel][receiver] (src/inject_extract.c:391-399).
"""
from __future__ import annotations

from typing import Sequence, Tuple

import numpy as np


def receiver_errors(d, dref, chans: Sequence[str], floor: float = 1e-3) -> Tuple[float, float]:
    """(largest amplitude error / channel scale, largest phase error in
    degrees) of d against dref, both [nch, nrec] complex."""
    nch = len(chans)
    d = np.asarray(d).reshape(nch, -1)
    dref = np.asarray(dref).reshape(nch, -1)
    kind_max = {}
    for c, nm in enumerate(chans):
        kind_max[nm[0]] = max(kind_max.get(nm[0], 0.0), float(np.abs(dref[c]).max()))
    amp, ph = 0.0, 0.0
    for c, nm in enumerate(chans):
        scale = max(float(np.abs(dref[c]).max()), floor * kind_max[nm[0]])
        if scale == 0:
            continue
        amp = max(amp, float(np.abs(d[c] - dref[c]).max()) / scale)
        sel = np.abs(dref[c]) > floor * scale
        if sel.any():
            ph = max(ph, float(np.degrees(np.abs(np.angle(d[c][sel] / dref[c][sel]))).max()))
    return amp, ph

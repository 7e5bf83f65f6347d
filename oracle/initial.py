"""CPU restatement of the channel's initial velocity (numpy).

TEST INFRASTRUCTURE ONLY: the engine's ``lbm_init_channel`` is checked
against it.  It follows initvel of
3DChannel_Decaying_HIT_Finite_Size_Moving_Particles/initial.f90:57-126 with
the constants of that program's para.f90:12-17 (visc, Rstar = 180,
ustar = 2 Rstar visc / nx, ystar = visc / ustar): u = w = 0 and, for the
nx/2 nodes nearest each wall (i = 1..nx/2 and its mirror nx + 1 - i),
y+ = (i - 1/2) / ystar, v = y+ ustar below y+ = 10.8, else
(ln(y+)/0.41 + 5) ustar.  The perturbation terms of the reference carry the
amplitude A9 = 0 and vanish.  Fields are (nz, ny, nx).
"""

from __future__ import annotations

import math

import numpy as np


def channel_loglaw(nx: int, ny: int, nz: int, visc: float):
    ustar = 2.0 * 180.0 * visc / float(nx)
    ystar = visc / ustar
    v = np.zeros(nx)
    for i in range(1, nx // 2 + 1):
        yplus = (float(i) - 0.5) / ystar
        if yplus < 10.8:
            u9 = yplus * ustar
        else:
            u9 = math.log(yplus) / 0.41 + 5.0
            u9 = u9 * ustar
        v[i - 1] = u9
        v[nx - i] = u9
    uy = np.broadcast_to(v[None, None, :], (nz, ny, nx)).copy()
    return np.zeros((nz, ny, nx)), uy, np.zeros((nz, ny, nx))

"""Host-side bookkeeping of the reference's solvent analyses whose sums over
particles run on the device (``Context.fourier_modes``, ``Context.vacf_*``):

* ``FourierAutocorr`` -- Fourier_Autocorr (star-polymers/lib/Analysis/Fourier_Autocorr.h):
  a window of ``entries`` samples of the three transverse modes; once it is
  full every sample adds Re(conj(m_j(oldest)) . m_j(oldest + lag)) per
  direction j; the result is that sum over the number of calculations;
* ``vacf_average`` / ``vacf_diffusion`` -- Vel_Autocorr_Fluid::calculate_average
  and ::value (star-polymers/lib/Analysis/Vel_Autocorr_Fluid.h), from the
  device's lag sums.
"""
from __future__ import annotations

import numpy as np


class FourierAutocorr:
    def __init__(self, entries: int, dt: float):
        self.entries = int(entries)
        self.dt = float(dt)
        self.window = []
        self.acc = np.zeros((3, self.entries))
        self.counter = 0

    def push(self, modes: np.ndarray) -> None:
        """modes: complex (3, 3), mode along x, y, z by velocity component."""
        self.window.append(np.asarray(modes, dtype=np.complex128))
        if len(self.window) > self.entries:
            self.window.pop(0)
        if len(self.window) == self.entries:
            first = self.window[0]
            for j in range(3):
                for lag in range(self.entries):
                    self.acc[j, lag] += np.real(np.vdot(first[j], self.window[lag][j]))
            self.counter += 1

    def result(self):
        """(times, autocorrelation (entries, 3)) as Fourier_Autocorr::print_result."""
        t = np.arange(self.entries) * self.dt
        return t, (self.acc / max(self.counter, 1)).T


def vacf_average(lag_sums: np.ndarray, calculations: int, n_particles: int) -> np.ndarray:
    """Vel_Autocorr_Fluid::calculate_average: per lag, the sum over particles of
    the accumulated products over the calculations, over the particles."""
    if calculations == 0:
        return np.zeros_like(np.asarray(lag_sums, dtype=np.float64))
    return np.asarray(lag_sums, dtype=np.float64) / calculations / n_particles


def vacf_diffusion(average: np.ndarray, dt: float, calculations: int) -> float:
    """Vel_Autocorr_Fluid::value(): sum of average * dt / calculations, over 3
    (the reference divides by the number of calculations a second time)."""
    if calculations == 0:
        return 0.0
    return float(np.sum(np.asarray(average) * dt / calculations) / 3.0)

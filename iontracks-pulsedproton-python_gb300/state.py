"""The run record: :class:`Result` and the per-step :class:`Diagnostics`.

Field for field the same record as pulsed_ion_chamber/state.py:24-110, so the
reference's writers (output.py) and its CLI consume a result from this backend
unchanged. The per-step tallies arrive from the device in one copy at the end
of a run instead of one scalar triple per step.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

__all__ = ["Result", "Diagnostics"]


@dataclass
class Result:
    config: object
    time_s: np.ndarray  # end-of-step time, s
    f_t: np.ndarray  # (injected - recombined) / injected so far
    ks: float  # 1 / f after full clearance (NaN when the run was cut short)
    positive_array: np.ndarray  # final density, (no_xy, no_xy, no_z_with_buffer)
    negative_array: np.ndarray
    n_positive: np.ndarray  # scored positive carriers at the end of each step
    n_negative: np.ndarray
    injected_positive: np.ndarray  # scored carriers created during each step
    injected_negative: np.ndarray
    recombination: np.ndarray  # scored pairs lost during each step
    track_density_xy: np.ndarray  # (no_xy, no_xy) track centres per column


class Diagnostics:
    """Per-step tallies of one run, filled from device arrays or step by step."""

    def __init__(self, config):
        steps = int(config.total_time_steps)
        self.injected = np.zeros(steps)
        self.recombined = np.zeros(steps)
        self.n_positive = np.zeros(steps)
        self.n_negative = np.zeros(steps)
        self.track_density_xy = np.zeros((int(config.no_xy), int(config.no_xy)))

    def count_tracks(self, xs: np.ndarray, ys: np.ndarray) -> None:
        """Add track centres to the column histogram (``int()`` floors)."""
        n = self.track_density_xy.shape[1]
        flat = xs.astype(np.int64) * n + ys.astype(np.int64)
        self.track_density_xy += np.bincount(flat, minlength=self.track_density_xy.size).reshape(
            self.track_density_xy.shape
        )

    def record(self, step, injected, recombined, total_positive, total_negative) -> None:
        self.injected[step] = injected
        self.recombined[step] = recombined
        self.n_positive[step] = total_positive
        self.n_negative[step] = total_negative

    def record_block(self, first_step: int, tallies: np.ndarray) -> None:
        """Store ``tallies[s] = (injected, recombined, n+, n-)`` for steps
        ``first_step .. first_step + len(tallies) - 1``."""
        s0, s1 = first_step, first_step + len(tallies)
        self.injected[s0:s1] = tallies[:, 0]
        self.recombined[s0:s1] = tallies[:, 1]
        self.n_positive[s0:s1] = tallies[:, 2]
        self.n_negative[s0:s1] = tallies[:, 3]

    def build_result(self, config, time_s, f_t, ks, positive_array, negative_array) -> Result:
        return Result(
            config=config,
            time_s=time_s,
            f_t=f_t,
            ks=ks,
            positive_array=positive_array,
            negative_array=negative_array,
            n_positive=self.n_positive,
            n_negative=self.n_negative,
            injected_positive=self.injected,
            injected_negative=self.injected.copy(),
            recombination=self.recombined,
            track_density_xy=self.track_density_xy,
        )


def collection_efficiency(injected: np.ndarray, recombined: np.ndarray, steps_completed: int) -> np.ndarray:
    """f(t) from per-step tallies, as the reference's drivers form it from
    running float64 totals (pulsed_ion_chamber/solver_numba.py:311, :333,
    :350): ``f = 1`` until something is injected, then ``(I - R) / I``. Steps
    past ``steps_completed`` keep 1.0, as in a run stopped early."""
    f_t = np.ones(len(injected))
    n = int(steps_completed)
    if n <= 0:
        return f_t
    # cumsum adds left to right, exactly the running float64 totals
    total_i = np.cumsum(np.asarray(injected[:n], dtype=np.float64))
    total_r = np.cumsum(np.asarray(recombined[:n], dtype=np.float64))
    with np.errstate(invalid="ignore", divide="ignore"):
        f = (total_i - total_r) / total_i
    f_t[:n] = np.where(total_i == 0.0, 1.0, f)
    return f_t

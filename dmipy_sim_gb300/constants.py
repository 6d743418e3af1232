"""Physical constants (the values of dmipy-sim's constants.py:6-30)."""
import numpy as np

# Proton gyromagnetic ratio, rad / (s T).
GAMMA = 267.513e6

# Default gradient slew rate, T/m/s: waveform constructors are slew-limited unless np.inf is passed.
DEFAULT_SLEW_RATE = 200.0


def resolve_slew(slew_rate):
    """Validate ``slew_rate``: a positive T/m/s value or np.inf (square lobes).

    Returns ``(slew_rate, is_square)``; None or non-positive values raise ValueError.
    """
    if slew_rate is None or not (slew_rate > 0):
        raise ValueError(
            "slew_rate must be a positive number (T/m/s) for a realistic slew-limited gradient, "
            "or np.inf for the idealized instantaneous (square) limit; got {!r}.".format(slew_rate))
    return slew_rate, (not np.isfinite(slew_rate))

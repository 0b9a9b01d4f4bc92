"""Comparison helpers for the reference's printed outputs (format 4E18.4)."""
import numpy as np


def printed_match(mine, gold, rel_floor=1e-10, full=None, units=0.6):
    """True where ``mine`` rounds to the 4 printed significant digits of ``gold``.

    E18.4 prints 0.dddd x 10^e, so the half-unit of the last digit is
    0.5e-4 * 10^e; 0.6e-4 leaves room for the last-digit rounding of the
    reference's own FP64 run.  Entries below ``rel_floor`` x max|full| are
    round-off noise in the reference (e.g. Re Tr G^< ~ 1e-14, or G^> where
    f = 1) and are skipped; ``full`` (default ``gold``) is the whole golden
    column the floor refers to.  ``units`` is the allowed distance in units of the
    last printed digit (0.6: the value rounds to the printed digits).
    """
    mine = np.asarray(mine, dtype=np.float64)
    gold = np.asarray(gold, dtype=np.float64)
    scale = np.where(gold != 0, 10.0 ** (np.floor(np.log10(np.abs(gold) + 1e-300)) + 1), 1.0)
    ok = np.abs(mine - gold) <= units * 1e-4 * scale
    ref = np.abs(np.asarray(gold if full is None else full)).max()
    noise = np.abs(gold) < rel_floor * ref
    return ok | noise

"""Physical constants of the propagation (Zandpack/td_constants.py:3-6)."""
HBAR = 6.582119569e-1  # eV * fs
ELECTRON_CHARGE = 1.0

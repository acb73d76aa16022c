"""Physical constants under the names the reference exports
(ufo/constants.py:8-13, re-exported by ufo/__init__.py:5).

The values are CODATA figures and the two radiation constants of the
synchrotron-radiation integrals (SLAC-1193):
  quantum_radiation_constant  C_q = 55 hbar c / (32 sqrt(3) m_e c^2), metres
  radiation_loss_constant     C_gamma / (2 pi), metres per GeV^3, so that
                              U0 [GeV] = radiation_loss_constant E[GeV]^4 I2
"""
speed_of_light = 2.99792458e8            # m/s
electron_mass = 0.51099895e6             # eV
electron_radius = 2.81794092e-15         # m
elementary_charge = 1.602176634e-19      # C
quantum_radiation_constant = 3.832e-13   # m
radiation_loss_constant = 14.085e-6      # m / GeV^3

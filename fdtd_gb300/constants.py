"""Physical constants and axis indices (same values as fdtd/constants.py:5-23)."""

from math import pi

c: float = 299792458.0
""" speed of light """

X: int = 0
Y: int = 1
Z: int = 2

mu0: float = 4e-7 * pi
""" vacuum permeability """

eps0: float = 1.0 / (mu0 * c ** 2)
""" vacuum permittivity """

eta0: float = mu0 * c
""" free space impedance """

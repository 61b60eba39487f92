"""Simulation-unit <-> SI field scaling (fdtd/conversions.py:32-45)."""

from math import sqrt

from . import constants as const


def simE_to_worldE(value):
    return value / sqrt(const.eps0)


def worldE_to_simE(value):
    return sqrt(const.eps0) * value


def simH_to_worldH(value):
    return value / sqrt(const.mu0)


def worldH_to_simH(value):
    return sqrt(const.mu0) * value

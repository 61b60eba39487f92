"""CPU oracle of the fdtd time step (test infrastructure only; see fdtd_oracle.py)."""

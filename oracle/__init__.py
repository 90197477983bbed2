"""CPU oracle package -- test infrastructure only (``fv_oracle``, ``operator_oracle``, ``ilu0_oracle.c``)."""

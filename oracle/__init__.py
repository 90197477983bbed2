"""CPU oracle package -- test infrastructure only (see ``fv_oracle`` and ``ilu0_ref``)."""

"""CPU oracle of the PNFFT hot path -- test infrastructure only (see pnfft_oracle.py)."""

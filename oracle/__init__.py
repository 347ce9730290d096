"""CPU oracle package (test infrastructure only; see scft_oracle.py)."""

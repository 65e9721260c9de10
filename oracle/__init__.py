"""CPU oracle (test infrastructure; see corr_oracle.py). Not part of the product."""

"""CPU oracle package: test infrastructure only (see bqa_oracle.py)."""

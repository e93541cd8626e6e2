"""CPU oracle of the SDGC recurrence -- test infrastructure only (see sdnn_oracle.c)."""

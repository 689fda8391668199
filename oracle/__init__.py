"""CPU oracle of the P3 step (test infrastructure; see p3_oracle.h)."""

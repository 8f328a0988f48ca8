"""CPU oracle of the SR particle-in-cell hot path (test infrastructure only)."""

"""CPU oracle of the split finite-volume patch update (test infrastructure only)."""

"""CPU oracle of the FARM polygon-join hot path (test infrastructure only)."""

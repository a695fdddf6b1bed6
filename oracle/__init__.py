"""CPU oracle of the DPLR apply / inverse path (test infrastructure only)."""

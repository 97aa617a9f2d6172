"""CPU oracle of the MPCD + active-colloid step (test infrastructure only)."""

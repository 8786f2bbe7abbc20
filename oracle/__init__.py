"""CPU oracle of the PSM lattice step -- test infrastructure, never product code."""

"""CPU oracle of the wavefront-series hot path (test infrastructure only)."""

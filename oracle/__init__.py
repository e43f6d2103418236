"""CPU oracle of the IB3D hot path (test infrastructure only)."""

"""CPU oracle of the planet hot path: test infrastructure only (parity unpinned)."""

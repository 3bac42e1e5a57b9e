"""CPU oracle of the enblend/enfuse hot path (test infrastructure only)."""

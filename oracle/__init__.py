"""CPU oracle of the block-IPT path (test infrastructure only)."""

"""CPU oracle of the interface-flux path (test infrastructure; never the product path)."""

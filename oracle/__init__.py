"""CPU oracle of the PaMO stage-2 path (test infrastructure: the checker, never the product)."""

"""CPU oracle of the batched block-tridiagonal solver (test infrastructure only)."""

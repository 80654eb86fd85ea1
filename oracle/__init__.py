"""CPU oracle for the blocked exact-kNN path (test infrastructure only; never imported by the product)."""

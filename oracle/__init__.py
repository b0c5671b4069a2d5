"""CPU oracle for the hex8 hot path (test infrastructure; never imported by the product)."""

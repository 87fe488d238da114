"""CPU oracles for parity tests (test infrastructure, never imported by the product)."""

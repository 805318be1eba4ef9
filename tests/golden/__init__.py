"""Golden fixtures of the parity tests and the scripts that made them."""

"""CPU oracle of the correlation scan (test infrastructure; see fftdock_oracle)."""

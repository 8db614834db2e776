"""CPU oracle of the radiosity path: test infrastructure only (see oracle.py)."""

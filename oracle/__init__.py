"""CPU oracle of the PBF step — test infrastructure only (see oracle/oracle.py)."""

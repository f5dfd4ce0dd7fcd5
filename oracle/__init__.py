"""TEST INFRASTRUCTURE ONLY: the CPU FP64 oracle of the focuser (see oracle.py)."""

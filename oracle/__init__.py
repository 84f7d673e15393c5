"""TEST INFRASTRUCTURE ONLY: the CPU oracle of the stepper (see oracle.py)."""

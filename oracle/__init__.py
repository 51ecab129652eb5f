"""CPU oracle package (test infrastructure): see pyoracle.py."""

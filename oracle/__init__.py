"""ORACLE — test infrastructure only (the checker). See pyoracle.py."""

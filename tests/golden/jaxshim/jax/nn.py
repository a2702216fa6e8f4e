"""Unused by the path; present because model.py imports it."""

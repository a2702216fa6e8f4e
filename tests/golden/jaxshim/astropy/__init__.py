"""Minimal astropy stand-in: units with SI scale factors and CODATA-2018 G."""

"""Substrate geometry generators (host numpy; inputs to ``set_solid``)."""

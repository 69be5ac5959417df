"""Import stub: ProjectQ's drawing helpers import this module by name."""

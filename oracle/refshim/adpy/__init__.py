"""Stand-in package for the empty adpy submodule of the reference (test infrastructure)."""

"""Stand-in: the oracle never reads or writes HDF5."""

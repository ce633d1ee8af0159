"""Stand-in: only the REGULAR_GRID mesh branch uses findiff; the oracle never takes it."""

"""GB300-native engine for FARM's polygon-join hot path."""

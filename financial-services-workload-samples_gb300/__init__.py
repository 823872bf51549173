"""GB300-native LMM swaption-portfolio Greeks engine (placeholder, filled in below)."""

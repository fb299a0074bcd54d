"""GB300-native se_e2_a descriptor hot path."""

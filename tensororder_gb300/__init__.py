"""GB300-native contraction backend for TensorOrder's Execution stage."""

"""GB300-native STCDB per-timestep co-occurrence pipeline."""

"""GB300-native (sm_103a) explicit residual-and-update loop of FiniteVolume."""

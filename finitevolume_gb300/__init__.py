"""GB300-native (sm_103a) explicit residual-and-update loop of FiniteVolume."""

__version__ = "0.1.0"

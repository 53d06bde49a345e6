"""GB300-native model-evaluation path of BBarolo 2's 3DFIT (GALMOD + beam + flux normalisation + log L)."""

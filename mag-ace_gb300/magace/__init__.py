"""GB300 implementation of the mag-ace potential evaluation (non-collinear
magnetic Atomic Cluster Expansion): Python helpers around libmagace.so."""

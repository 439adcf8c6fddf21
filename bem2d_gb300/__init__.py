"""bem2d_gb300: GB300-native Galerkin assembly and dense solves for bem2d."""

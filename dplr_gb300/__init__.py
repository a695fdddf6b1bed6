"""GB300-native DPLR: PLR (HODLR) apply and solve on sm_103a."""

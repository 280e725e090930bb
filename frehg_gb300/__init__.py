"""GB300-native (sm_103a) Richards-equation groundwater step of zLi90/frehg."""

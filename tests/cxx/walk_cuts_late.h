// Uneven cuts for the split test (the last part small).
#define MBPOL_WALK_CUTS_3B {0.37, 0.80}
#define MBPOL_WALK_CUTS_2B {0.20, 0.95}

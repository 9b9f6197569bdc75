"""sffg: GB300-native generalized-Born energy/gradient engine with the C API
of dacase/nabc's SFF library (mm_options / mme_init_sff / mme / md /
conjgrad).  The compute path is libsffg.so (hand-written sm_103a CUDA);
this package only builds and binds it."""

/* ozaki_model.c -- host model of the Ozaki-scheme slicing (filled in with the
 * tensor-core form).  TEST INFRASTRUCTURE ONLY. */
int orc_ozaki_model_version(void) { return 0; }

// Mixed-form modified Picard step on the device (not in reference).
#pragma once
struct frehg_re;
static int picard_step(frehg_re* re) {
  (void)re;
  fg::set_error("the Picard scheme is not built in this version");
  return FREHG_ERR_UNSUPPORTED;
}

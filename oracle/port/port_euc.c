/*
 * ORACLE -- test infrastructure, never part of the product.
 * C restatement of the Eucclhyd scheme (eucclhyd_remap/); filled in below.
 */
#include <stdlib.h>

#include "port_internal.h"

int port_euc_setup(port_run* R) {
  (void)R;
  port_set_error("Eucclhyd scheme not available in the C restatement yet");
  return -1;
}
void port_euc_cycle(port_run* R) { R->done = 1; }
void port_euc_free(port_run* R) { free(R->euc); R->euc = NULL; }

/* A plain C99 client of libfheg: the header compiles as C, every host-only
 * entry point links and answers. Built and run by tests/test_abi_host.py. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "fheg.h"

int main(void) {
  uint64_t p = 0, root = 0;
  uint32_t bl = 0;
  if (strncmp(fheg_version(), "fheg", 4) != 0) return 1;
  if (fheg_generate_prime(62, 2 * 16384, (uint64_t)1 << 62, &p) != FHEG_OK) return 2;
  if (p != 4611686018427322369ULL) return 3;
  if (!fheg_supports_ntt(p, 16384)) return 4;
  if (fheg_ntt_default_root(p, 16384, &root) != FHEG_OK || root == 0) return 5;
  if (fheg_ntt_plan_get(14, &bl) != FHEG_OK || bl != 12) return 6;
  if (fheg_ntt_plan_set(14, 11) != FHEG_ERR_INVALID_ARGUMENT) return 7;
  if (strlen(fheg_last_error()) == 0) return 8;
  if (strcmp(fheg_status_string(FHEG_ERR_TIMEOUT), "timeout") != 0) return 9;
  printf("ok %llu %llu\n", (unsigned long long)p, (unsigned long long)root);
  return 0;
}

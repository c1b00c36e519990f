/* Internal declarations shared by the host C file and the CUDA files. */
#ifndef VG_INTERNAL_H
#define VG_INTERNAL_H
#include "../../include/vegas_gb300.h"

/* Per-device host caches (forked streams, the no-alloc scratch address) are
 * indexed by device ordinal below this bound. */
#define VG_MAX_DEVICES 64

#ifdef __cplusplus
extern "C" {
#endif
/* Record an error message (thread-local) and return `code`. */
int vg_fail(int code, const char *fmt, ...);
/* Clear the thread-local error message. */
void vg_clear_error(void);
#ifdef __cplusplus
}
#endif
#endif

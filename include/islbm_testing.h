/* islbm_testing.h - hooks for testing the failure path of the step kernels.
 *
 * No reference counterpart. The tiled step kernel waits for its shared-memory copies with
 * bounded waits (about a second); when one runs out, the kernel records the fault in the
 * solve's controller, stops starting copies, waits (bounded again) for those in flight and
 * completes, so the device context stays usable; islbm_sync then returns ISLBM_ERR_CUDA.
 * This hook makes such a wait run out without faulting anything: the copies of one plane are
 * simply never started.
 */
#ifndef ISLBM_TESTING_H
#define ISLBM_TESTING_H

#include "islbm.h"

#ifdef __cplusplus
extern "C" {
#endif

/* From the next islbm_step on, the tiled kernel skips the copies of wall-normal plane `plane`
 * (0 <= plane < NZ); -1 turns the drill off. The solve's state is undefined afterwards. */
ISLBM_API int islbm_fault_drill(islbm_handle *h, int plane);

#ifdef __cplusplus
}
#endif
#endif

/*
 * GpuPixelSearchByTriplet.h -- the reference's C++ entry points, same names,
 * signatures and argument meaning (GpuPixelSearchByTriplet.h:12-29,
 * KernelInvoker.h:27-31, Tools.h:47 of dcampora/cl_forward), implemented on
 * the C ABI in velo_search.h by libclforward_gb300.so.
 *
 *   input[e]   one event blob (layout in velo_search.h)
 *   output[e]  count * sizeof(Track) bytes of Track records (100 B each);
 *              hits are event-local indices into the x-sorted hit arrays.
 *
 * Error behaviour follows the reference: a device or input error prints a
 * message on stderr and ends the process with exit(-1) (Tools.h:27-34); the
 * return value is 0.  Callers that want status codes use velo_search().
 */
#ifndef CL_FORWARD_GB300_GPUPIXELSEARCHBYTRIPLET_H
#define CL_FORWARD_GB300_GPUPIXELSEARCHBYTRIPLET_H

#include <stdint.h>

#include <vector>

/* Standalone entry: sorts each module's hits by x, then searches.  The sort
 * runs on the GPU, in chunks of at most 16000 events, with the reference's
 * permutation; the sorted bytes are written back into the input (through the
 * const reference, as the reference's host sort leaves them). */
int independent_execute(const std::vector<std::vector<uint8_t> >& input,
                        std::vector<std::vector<uint8_t> >& output);

/* Prints the number of output entries (GpuPixelSearchByTriplet.cpp:24-27). */
void independent_post_execute(const std::vector<std::vector<uint8_t> >& output);

/* Framework entry: input must already be x-sorted per module; silent. */
int gpuPixelSearchByTriplet(const std::vector<const std::vector<uint8_t>*>& input,
                            std::vector<std::vector<uint8_t> >& output);

/* Common path: resizes output to input.size() and searches in chunks of at
 * most 16000 events (GpuPixelSearchByTriplet.cpp:44-65). */
int gpuPixelSearchByTripletInvocation(const std::vector<const std::vector<uint8_t>*>& input,
                                      std::vector<std::vector<uint8_t> >& output);

/* Searches input[startingEvent, startingEvent + eventsToProcess) and resizes
 * output[startingEvent + i] to its tracks (KernelInvoker.cpp:14-275). */
int invokeParallelSearch(const int startingEvent, const int eventsToProcess,
                         const std::vector<const std::vector<uint8_t>*>& input,
                         std::vector<std::vector<uint8_t> >& output);

/* Per-module x-sort of every event, in place (Tools.cpp:46-66). */
void preorder_by_x(std::vector<const std::vector<uint8_t>*>& input);

#endif

/* voss.h -- error codes and memory helpers of the voss C ABI.
 *
 * Drop-in for the reference's library/include/voss/voss.h:1-31: the same
 * codes, the same two message functions and the same free function, so a
 * binding written against the reference links unchanged.
 */
#ifndef VOSS_H
#define VOSS_H

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes of every int-returning voss function (voss.h:9-16). */
#define VOSS_OK                     0
#define VOSS_ERR_INVALID_N          1
#define VOSS_ERR_OUT_OF_RANGE       2
#define VOSS_ERR_NO_CUDA            3
#define VOSS_ERR_OUT_OF_MEMORY      4
#define VOSS_ERR_CUDA               5
#define VOSS_ERR_INVALID_ARG        6
#define VOSS_ERR_INTERNAL           7

/* Short fixed text for a code (replaces error.cpp:20-31). */
const char* voss_strerror(int code);

/* Detail of the last failure on the calling thread (replaces
 * error.cpp:10-18; thread-local, overwritten by the next failure). */
const char* voss_get_last_error(void);

/* Release an array returned by a voss function; NULL is a no-op
 * (replaces alloc.cpp:7-9: arrays come from malloc). */
void voss_free(void* ptr);

#ifdef __cplusplus
}
#endif

#endif /* VOSS_H */

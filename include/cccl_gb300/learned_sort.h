/* Learned-partition radix sort.
 *
 * No counterpart in the reference: a second form of cccl_device_radix_sort
 * (c/parallel/include/cccl/c/radix_sort.h:110-124) with the same run signature, the same
 * output bit for bit (key order including -0.0/+0.0 and NaN patterns, stable order of the
 * values of equal keys) and the same returned selector. A caller switches by calling
 * cccl_gb300_learned_sort where it called cccl_device_radix_sort.
 *
 * How it sorts: a two-level piecewise-linear model of the keys' distribution is fitted by
 * least squares on a 65536-key sample ranked by the plain radix sort; every key is routed
 * to one of about num_items/4096 buckets by stable partition passes on the model's bucket
 * id (one pass per 8 bits of bucket id, so the number of passes over HBM does not grow with
 * the key width); every bucket is then sorted in shared memory, and a bucket too large for
 * that is sorted by the plain radix passes. The bucket id never decreases as the key grows,
 * so a poor model costs time, never correctness.
 *
 * Keys: 4- and 8-byte integer and floating-point types; values: none, 4 or 8 bytes. Inputs
 * the learned path does not take (fewer than 2^20 keys, a bit window narrower than the key,
 * buffers not 16-byte aligned) are sorted by the plain radix sort. So are inputs the model
 * predicts the partition cannot pay for: after the fit, a kernel checks how much of the
 * sorted sample lies in buckets predicted to overflow the bucket sort, and above half
 * (near-constant keys, heavy duplicates) the plain sort runs instead. The choice is made on
 * the device, without a host synchronisation, and the result and selector are the same.
 *
 * Before that, a cost model on the host compares bytes moved: the partition passes plus the
 * bucket sort against the plain sort's one pass per key byte, with the learned kernels
 * counted at 0.7 of the plain passes' bandwidth (measured on GB300). It sends 4-byte keys to
 * the plain sort (3 learned passes cannot beat 4 plain ones there) and takes 8-byte keys.
 * cccl_gb300_learned_sort_set_route(build, CCCL_GB300_LEARNED_ROUTE_ALWAYS) switches the
 * cost model off for a build (every qualifying input takes the learned kernels).
 */
#pragma once

#ifndef CCCL_C_EXPERIMENTAL
#  error "C exposure is experimental and subject to change. Define CCCL_C_EXPERIMENTAL to acknowledge this notice."
#endif

#include <cuda.h>

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#include <cccl/c/extern_c.h>
#include <cccl/c/types.h>
#include <cccl_gb300/sort_trace.h>

CCCL_C_EXTERN_C_BEGIN

typedef struct cccl_gb300_learned_sort_build_result_t
{
  int cc;
  cccl_type_info key_type;
  cccl_type_info value_type;
  cccl_sort_order_t order;
  CUlibrary radix_library;     /* plain radix kernels: the sample sort and the fallback */
  CUlibrary segmented_library; /* bucket sort */
  CUlibrary learned_library;   /* sample, fit, histogram, partition pass, bucket bounds */
  void* setup;                 /* kernel handles and tile shapes, owned by the build result */
  size_t setup_size;
} cccl_gb300_learned_sort_build_result_t;

/* What the last run did, read back from its temporary storage. */
typedef struct cccl_gb300_learned_sort_stats_t
{
  int learned;             /* 0: the plain radix sort ran (input not taken, or routed to it on the device) */
  int bucket_log2;         /* log2 of the number of buckets */
  int partition_passes;    /* stable passes on the bucket id */
  uint32_t block_buckets;  /* non-empty buckets sorted in shared memory */
  uint32_t device_buckets; /* buckets handed to the plain radix passes */
  uint64_t device_items;   /* keys in those buckets */
} cccl_gb300_learned_sort_stats_t;

/* Arguments as cccl_device_radix_sort_build's (radix_sort.h:63-75) without the source and
 * header paths: the kernels are precompiled for sm_103a (cc_major.cc_minor must be 10.3). */
CCCL_GB300_API CUresult cccl_gb300_learned_sort_build(
  cccl_gb300_learned_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t input_keys_it,
  cccl_iterator_t input_values_it,
  int cc_major,
  int cc_minor);

/* Arguments and results as cccl_device_radix_sort (radix_sort.h:110-124). */
CCCL_GB300_API CUresult cccl_gb300_learned_sort(
  cccl_gb300_learned_sort_build_result_t build,
  void* d_temp_storage,
  size_t* temp_storage_bytes,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  cccl_op_t decomposer,
  uint64_t num_items,
  int begin_bit,
  int end_bit,
  bool is_overwrite_okay,
  int* selector,
  CUstream stream);

/* Reads the counters of a finished run (same arguments as the run). Synchronous: the run
 * must be complete, e.g. after cuStreamSynchronize on its stream. */
CCCL_GB300_API CUresult cccl_gb300_learned_sort_stats(
  cccl_gb300_learned_sort_build_result_t build,
  void* d_temp_storage,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  uint64_t num_items,
  int begin_bit,
  int end_bit,
  bool is_overwrite_okay,
  cccl_gb300_learned_sort_stats_t* stats);

/* Route policy of a build: CCCL_GB300_LEARNED_ROUTE_COST_MODEL (the default after
 * cccl_gb300_learned_sort_build) or CCCL_GB300_LEARNED_ROUTE_ALWAYS. */
#define CCCL_GB300_LEARNED_ROUTE_COST_MODEL 0
#define CCCL_GB300_LEARNED_ROUTE_ALWAYS 1
CCCL_GB300_API CUresult cccl_gb300_learned_sort_set_route(cccl_gb300_learned_sort_build_result_t* build, int route);

CCCL_GB300_API CUresult cccl_gb300_learned_sort_cleanup(cccl_gb300_learned_sort_build_result_t* build);

CCCL_C_EXTERN_C_END

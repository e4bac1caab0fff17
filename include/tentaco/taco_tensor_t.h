/*
 * taco_tensor_t -- the tensor descriptor every entry point of libtentaco_gb300 takes.
 *
 * Same field order, types and meaning as the reference's descriptor
 * (taco_tensor_t.h:6-15 of zhang677/tenTACO), so that a caller compiled against
 * the reference header passes its structs to this library unchanged:
 *
 *   order          number of modes
 *   dimensions     per-mode sizes (dimensions[1] of a dense factor/output is the rank R)
 *   csize          component size in bytes (informational)
 *   mode_ordering  storage order of the modes (informational; CSF levels follow it)
 *   mode_types     taco_mode_dense / taco_mode_sparse per level
 *   indices        indices[level][0] = pos, indices[level][1] = crd (int32)
 *   vals           value array (float on the GPU surface)
 *   vals_size      number of entries in vals (informational)
 *
 * CSF convention accepted by the library (level 0 = root):
 *   - dense root:       mode_types[0] == taco_mode_dense, or indices[0] == NULL.
 *                       indices[1][0] (pos) has dimensions[0]+1 entries; empty
 *                       rows are allowed.
 *   - compressed root:  indices[0] = {pos = [0, n0], crd = row ids (n0 entries)},
 *                       as produced by the reference's compress_top_level
 *                       (ds.h:426-436); indices[1][0] then has n0+1 entries.
 *   Inner levels l >= 1: indices[l][0] has (#fibers at level l-1)+1 entries,
 *   indices[l][1] has (#fibers at level l) entries; inner fibers are non-empty.
 */
#ifndef TENTACO_TACO_TENSOR_T_H
#define TENTACO_TACO_TENSOR_T_H
#include <stdint.h>

#ifndef TACO_TENSOR_T_DEFINED
#define TACO_TENSOR_T_DEFINED
typedef enum { taco_mode_dense, taco_mode_sparse } taco_mode_t;

typedef struct taco_tensor_t {
  int32_t      order;
  int32_t*     dimensions;
  int32_t      csize;
  int32_t*     mode_ordering;
  taco_mode_t* mode_types;
  int32_t***   indices;
  float*       vals;
  int32_t      vals_size;
} taco_tensor_t;
#endif

#endif /* TENTACO_TACO_TENSOR_T_H */

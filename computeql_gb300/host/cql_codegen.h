/*
 * cql_codegen.h - the code generator's entry points inside the operator layer.
 */
#ifndef CQL_CODEGEN_H
#define CQL_CODEGEN_H

#include <stddef.h>
#include <stdint.h>

#include "cqlops.h"

/* one comparison of a column with a literal in a batched query: the literal's index in the query's
   constant pool, the comparison opcode and the column type; the thresholds are worked out per query */
typedef struct
{
  uint32_t const_index, op, col_type, pad;
} CqlBatchSite;

/* The program as one boolean expression over raw row k of the column registers r<slot>[k], its
   comparisons with literals reading the query's thresholds T<site> (copies of TH[site] the caller
   declares; cql_bi / cql_bf, and cql_bk over kd<slot>[k], the order keys of an f64 column the caller
   computes once per row) and any other literal QC[index]. Lists the sites and the slot types the expression reads. Returns 0 with
   `why` when the program cannot be batched (strings, 64-bit integer comparisons). */
int cql_codegen_batch_predicate(const CqlProgram* prog, CqlBatchSite* sites, uint32_t site_cap, uint32_t* site_count, int* slot_type,
                                char** expr, char* why, size_t why_cap);

#endif

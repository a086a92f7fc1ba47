/*
 * cql_program.c - WHERE conditions to the reference's scan bytecode.
 *
 * Mirrors qe_bytecode_program_build / qe_compile_condition (src/query_exec/query_exec.c:204-548) and
 * their helpers (:1-200): the same opcodes (query_exec.h:58-81), the same f64 constant pool as
 * (lo, hi) words, the same 4-byte aligned string pool, the same slot allocation (a raw string
 * column takes a data and an offsets slot, dictionary codes one U32 slot), IN lists expanded to an
 * OR chain of '=' (an AND chain of '!=' for NOT IN), at most 32 items.
 *
 * The condition arrives as an s-expression over named columns instead of the reference's IR tree:
 *   (and A B) (or A B) (= a 5) (!= a 5) (< a 2.5) (<= ..) (> ..) (>= ..) (in a 1 2 3) (not_in a 1 2)
 *   (is_null a) (is_not_null a) (contains s 'text') true false
 *   (> (similarity s 'text') 0.4) (<= (edit_distance s 'text') 2)   - fuzzy search, the score reported per row
 * Literals: numbers, or 'quoted' strings for string columns.
 */
#include "cqlops.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

enum
{
  OP_PUSH_TRUE = 0, OP_LOAD_NUM_COL = 1, OP_PUSH_CONST = 2, OP_CMP_EQ = 3, OP_CMP_NE = 4, OP_CMP_LT = 5, OP_CMP_GT = 6,
  OP_CMP_LE = 7, OP_CMP_GE = 8, OP_AND = 9, OP_OR = 10, OP_STR_EQ = 11, OP_STR_CONTAINS = 12, OP_HALT = 13, OP_PUSH_FALSE = 14,
  OP_TRIGRAM_SIM = 15, OP_EDIT_DISTANCE = 16, OP_STR_NE = 17, OP_STR_LT = 18, OP_STR_GT = 19, OP_STR_LE = 20, OP_STR_GE = 21,
};

#define IN_LIST_GPU_MAX_ITEMS 32

/* ---- s-expression reader ---- */

typedef struct Node Node;
struct Node
{
  int is_list;
  char atom[256];
  int quoted;
  Node* first;
  Node* next;
};

typedef struct
{
  const char* s;
  size_t i;
  int failed;
} Reader;

static void skip_ws(Reader* r)
{
  while (r->s[r->i] && isspace((unsigned char)r->s[r->i])) r->i++;
}

static Node* read_node(Reader* r)
{
  skip_ws(r);
  char c = r->s[r->i];
  if (!c || c == ')')
  {
    r->failed = 1;
    return NULL;
  }
  Node* n = (Node*)calloc(1, sizeof(Node));
  if (c == '(')
  {
    r->i++;
    n->is_list = 1;
    Node** tail = &n->first;
    for (;;)
    {
      skip_ws(r);
      if (r->s[r->i] == ')')
      {
        r->i++;
        break;
      }
      if (!r->s[r->i])
      {
        r->failed = 1;
        break;
      }
      Node* child = read_node(r);
      if (!child) break;
      *tail = child;
      tail = &child->next;
    }
    return n;
  }
  if (c == '\'')
  {
    r->i++;
    size_t k = 0;
    while (r->s[r->i] && r->s[r->i] != '\'' && k + 1 < sizeof(n->atom)) n->atom[k++] = r->s[r->i++];
    if (r->s[r->i] != '\'') r->failed = 1;
    else r->i++;
    n->quoted = 1;
    return n;
  }
  size_t k = 0;
  while (r->s[r->i] && !isspace((unsigned char)r->s[r->i]) && r->s[r->i] != '(' && r->s[r->i] != ')' && k + 1 < sizeof(n->atom))
    n->atom[k++] = r->s[r->i++];
  return n;
}

static void free_node(Node* n)
{
  while (n)
  {
    Node* next = n->next;
    free_node(n->first);
    free(n);
    n = next;
  }
}

/* ---- program building (qe_bytecode_emit, qe_add_numeric_const, qe_add_string_const, qe_bind_column) ---- */

typedef struct
{
  CqlProgram* prog;
  const CqlColumn* columns;
  const char* const* names;
  uint32_t column_count;
} Ctx;

static void fail(CqlProgram* p, const char* why)
{
  if (!p->error[0]) snprintf(p->error, sizeof(p->error), "%s", why);
}

static void emit(CqlProgram* p, uint32_t w)
{
  if (p->word_count >= CQLOPS_MAX_WORDS)
  {
    fail(p, "bytecode program exceeded its word limit");
    return;
  }
  p->words[p->word_count++] = w;
}

static uint32_t add_const(CqlProgram* p, double v)
{
  if (p->const_count >= CQLOPS_MAX_CONSTS)
  {
    fail(p, "bytecode program exceeded its constant limit");
    return 0;
  }
  uint64_t bits;
  memcpy(&bits, &v, sizeof(bits));
  uint32_t index = p->const_count++;
  p->consts[index * 2 + 0] = (uint32_t)(bits & 0xffffffffu);
  p->consts[index * 2 + 1] = (uint32_t)(bits >> 32);
  return index;
}

static void add_string(CqlProgram* p, const char* s, uint32_t* out_word_offset, uint32_t* out_len)
{
  uint32_t len = (uint32_t)strlen(s);
  uint32_t aligned = (p->str_pool_size + 3u) & ~3u;
  if (aligned + len > CQLOPS_MAX_STR_POOL)
  {
    fail(p, "string constant pool exhausted");
    *out_word_offset = 0;
    *out_len = 0;
    return;
  }
  memcpy(p->str_pool + aligned, s, len);
  p->str_pool_size = aligned + len;
  *out_word_offset = aligned / 4;
  *out_len = len;
}

static int find_column(Ctx* c, const char* name)
{
  for (uint32_t i = 0; i < c->column_count; i++)
  {
    if (c->names[i] && strcmp(c->names[i], name) == 0) return (int)i;
  }
  return -1;
}

/* binds column `index` (dict codes when use_dict); returns the binding number or -1 */
static int bind(Ctx* c, uint32_t index, int use_dict)
{
  CqlProgram* p = c->prog;
  for (uint32_t b = 0; b < p->binding_count; b++)
  {
    if (p->binding_column[b] == index && p->binding_dict[b] == (uint32_t)use_dict) return (int)b;
  }
  if (p->binding_count >= CQLOPS_MAX_BINDINGS)
  {
    fail(p, "exceeded max column bindings");
    return -1;
  }
  const CqlColumn* col = &c->columns[index];
  uint32_t slots = (col->type == CQLOPS_TYPE_STRING8 && !use_dict) ? 2 : 1;
  if (p->next_slot + slots > CQLOPS_MAX_BINDINGS)
  {
    fail(p, "exceeded available column slots");
    return -1;
  }
  uint32_t b = p->binding_count++;
  p->binding_column[b] = index;
  p->binding_type[b] = use_dict ? CQLOPS_TYPE_U32 : col->type;
  p->binding_slot[b] = p->next_slot;
  p->binding_dict[b] = (uint32_t)use_dict;
  p->next_slot += slots;
  return (int)b;
}

/* A string column with a dictionary is bound as its U32 codes (qe_bind_column_dict_codes). */
int cqlops_program_bind(CqlProgram* prog, const CqlColumn* columns, uint32_t column_index)
{
  Ctx c = { prog, columns, NULL, column_index + 1 };
  int use_dict = columns[column_index].type == CQLOPS_TYPE_STRING8 && columns[column_index].dict != NULL;
  int b = bind(&c, column_index, use_dict);
  return b < 0 ? -1 : (int)prog->binding_slot[b];
}

static int is_number(const char* s, double* out)
{
  char* end = NULL;
  double v = strtod(s, &end);
  if (end == s || *end) return 0;
  *out = v;
  return 1;
}

static uint32_t cmp_opcode(const char* op)
{
  if (!strcmp(op, "=") || !strcmp(op, "==")) return OP_CMP_EQ;
  if (!strcmp(op, "!=")) return OP_CMP_NE;
  if (!strcmp(op, "<=")) return OP_CMP_LE;
  if (!strcmp(op, ">=")) return OP_CMP_GE;
  if (!strcmp(op, "<")) return OP_CMP_LT;
  if (!strcmp(op, ">")) return OP_CMP_GT;
  return 0;
}

/* qe_compile_load_value (query_exec.c:77-100) */
static void load_value(Ctx* c, Node* n)
{
  CqlProgram* p = c->prog;
  double v;
  if (!n->is_list && !n->quoted && is_number(n->atom, &v))
  {
    emit(p, OP_PUSH_CONST);
    emit(p, add_const(p, v));
    return;
  }
  int ci = (!n->is_list && !n->quoted) ? find_column(c, n->atom) : -1;
  if (ci < 0)
  {
    fail(p, "unknown column or malformed value");
    emit(p, OP_PUSH_CONST);
    emit(p, add_const(p, 0.0));
    return;
  }
  int b = bind(c, (uint32_t)ci, 0);
  if (b < 0)
  {
    emit(p, OP_PUSH_CONST);
    emit(p, add_const(p, 0.0));
    return;
  }
  emit(p, OP_LOAD_NUM_COL);
  emit(p, (p->binding_type[b] << 8) | (p->binding_slot[b] & 0xffu));
}

static int dict_code(const CqlDict* d, const char* value, uint32_t* out)
{
  size_t len = strlen(value);
  for (uint32_t i = 0; i < d->count; i++)
  {
    uint32_t a = d->offsets[i], b = d->offsets[i + 1];
    if (b - a == len && memcmp(d->bytes + a, value, len) == 0)
    {
      *out = i;
      return 1;
    }
  }
  return 0;
}

static void compile(Ctx* c, Node* n);

#define FUZZY_MAX_NEEDLE_LEN 64

static void compile_comparison(Ctx* c, const char* op, Node* left, Node* right)
{
  CqlProgram* p = c->prog;
  /* fuzzy search: (op (similarity col 'term') threshold), (op (edit_distance col 'term') threshold)
     (:307-349): the score is compared, and also reported per matching row */
  if (left->is_list && left->first && !left->first->is_list &&
      (!strcmp(left->first->atom, "similarity") || !strcmp(left->first->atom, "edit_distance")))
  {
    int is_distance = !strcmp(left->first->atom, "edit_distance");
    Node* col_arg = left->first->next;
    Node* needle = col_arg ? col_arg->next : NULL;
    int ci = col_arg && !col_arg->is_list && !col_arg->quoted ? find_column(c, col_arg->atom) : -1;
    uint32_t cmp = cmp_opcode(op);
    if (ci < 0 || c->columns[ci].type != CQLOPS_TYPE_STRING8 || !needle || !needle->quoted || !cmp || (c->columns[ci].dict && !c->columns[ci].offsets))
    {
      fail(p, "similarity() / edit_distance() take a raw string column, a string literal and a comparison");
      emit(p, OP_PUSH_TRUE);
      return;
    }
    int b = bind(c, (uint32_t)ci, 0);
    if (b < 0)
    {
      emit(p, OP_PUSH_TRUE);
      return;
    }
    /* a needle longer than the kernels' limit is cut to it (QE_*_MAX_NEEDLE_LEN, 64 bytes by default) */
    char cut[FUZZY_MAX_NEEDLE_LEN + 1];
    snprintf(cut, sizeof(cut), "%s", needle->atom);
    uint32_t wo = 0, len = 0;
    add_string(p, cut, &wo, &len);
    emit(p, is_distance ? OP_EDIT_DISTANCE : OP_TRIGRAM_SIM);
    emit(p, p->binding_slot[b]);
    emit(p, wo);
    emit(p, len);
    p->has_score_output = is_distance ? 2u : 1u;
    load_value(c, right);
    emit(p, cmp);
    return;
  }
  /* string column op 'literal' (:358-455) */
  int li = (!left->is_list && !left->quoted) ? find_column(c, left->atom) : -1;
  if (li >= 0 && c->columns[li].type == CQLOPS_TYPE_STRING8 && right->quoted)
  {
    int is_contains = !strcmp(op, "contains");
    uint32_t cmp = cmp_opcode(op);
    if (!is_contains && !cmp)
    {
      fail(p, "unsupported string operator");
      emit(p, OP_PUSH_TRUE);
      return;
    }
    const CqlColumn* col = &c->columns[li];
    /* dictionary codes are assigned in insert order: only = and != can use them */
    if ((cmp == OP_CMP_EQ || cmp == OP_CMP_NE) && col->dict)
    {
      uint32_t code = 0;
      if (!dict_code(col->dict, right->atom, &code))
      {
        /* a literal absent from the dictionary matches no row for '=', every row for '!=' */
        emit(p, cmp == OP_CMP_NE ? OP_PUSH_TRUE : OP_PUSH_FALSE);
        return;
      }
      int b = bind(c, (uint32_t)li, 1);
      if (b < 0)
      {
        emit(p, OP_PUSH_TRUE);
        return;
      }
      emit(p, OP_LOAD_NUM_COL);
      emit(p, (p->binding_type[b] << 8) | (p->binding_slot[b] & 0xffu));
      emit(p, OP_PUSH_CONST);
      emit(p, add_const(p, (double)code));
      emit(p, cmp);
      return;
    }
    if (col->dict && !col->offsets)
    {
      fail(p, "a dictionary-coded column without raw strings takes only = and !=");
      emit(p, OP_PUSH_TRUE);
      return;
    }
    uint32_t opcode = OP_STR_EQ;
    if (is_contains) opcode = OP_STR_CONTAINS;
    else if (cmp == OP_CMP_NE) opcode = OP_STR_NE;
    else if (cmp == OP_CMP_LT) opcode = OP_STR_LT;
    else if (cmp == OP_CMP_GT) opcode = OP_STR_GT;
    else if (cmp == OP_CMP_LE) opcode = OP_STR_LE;
    else if (cmp == OP_CMP_GE) opcode = OP_STR_GE;
    int b = bind(c, (uint32_t)li, 0);
    if (b < 0)
    {
      emit(p, OP_PUSH_TRUE);
      return;
    }
    uint32_t wo = 0, len = 0;
    add_string(p, right->atom, &wo, &len);
    emit(p, opcode);
    emit(p, p->binding_slot[b]);
    emit(p, wo);
    emit(p, len);
    return;
  }
  uint32_t cmp = cmp_opcode(op);
  if (!cmp)
  {
    fail(p, "unsupported comparison operator");
    emit(p, OP_PUSH_TRUE);
    return;
  }
  /* generic numeric comparison (:541-545) */
  load_value(c, left);
  load_value(c, right);
  emit(p, cmp);
}

static void compile(Ctx* c, Node* n)
{
  CqlProgram* p = c->prog;
  if (!n)
  {
    emit(p, OP_PUSH_TRUE);
    return;
  }
  if (!n->is_list)
  {
    if (!strcmp(n->atom, "true"))
    {
      emit(p, OP_PUSH_TRUE);
      return;
    }
    if (!strcmp(n->atom, "false"))
    {
      emit(p, OP_PUSH_FALSE);
      return;
    }
    /* a bare column or literal as a predicate: nonzero is true (:207-213) */
    load_value(c, n);
    return;
  }
  Node* opn = n->first;
  if (!opn || opn->is_list)
  {
    fail(p, "malformed condition");
    emit(p, OP_PUSH_TRUE);
    return;
  }
  const char* op = opn->atom;
  Node* left = opn->next;
  Node* right = left ? left->next : NULL;
  if (!strcmp(op, "and") || !strcmp(op, "or"))
  {
    if (!left || !right)
    {
      fail(p, "and/or take two operands");
      emit(p, OP_PUSH_TRUE);
      return;
    }
    compile(c, left);
    compile(c, right);
    emit(p, !strcmp(op, "and") ? OP_AND : OP_OR);
    /* more operands fold left, as a chain of binary nodes would */
    for (Node* more = right->next; more; more = more->next)
    {
      compile(c, more);
      emit(p, !strcmp(op, "and") ? OP_AND : OP_OR);
    }
    return;
  }
  if (!strcmp(op, "is_null") || !strcmp(op, "is_not_null"))
  {
    /* the columns this path takes have no NULL flags: IS NULL is false, IS NOT NULL true (:233-246) */
    if (!strcmp(op, "is_not_null")) emit(p, OP_PUSH_TRUE);
    else
    {
      emit(p, OP_PUSH_CONST);
      emit(p, add_const(p, 0.0));
    }
    return;
  }
  if (!strcmp(op, "in") || !strcmp(op, "not_in"))
  {
    int is_not = !strcmp(op, "not_in");
    if (!left)
    {
      fail(p, "in needs a column and a list");
      emit(p, OP_PUSH_FALSE);
      return;
    }
    uint32_t items = 0;
    for (Node* it = right; it; it = it->next) items++;
    if (items == 0)
    {
      emit(p, is_not ? OP_PUSH_TRUE : OP_PUSH_FALSE);
      return;
    }
    if (left->is_list || items > IN_LIST_GPU_MAX_ITEMS)
    {
      p->requires_cpu_scan = 1;
      fail(p, "IN list too long for GPU bytecode");
      emit(p, OP_PUSH_TRUE);
      return;
    }
    int first = 1;
    for (Node* it = right; it; it = it->next)
    {
      compile_comparison(c, is_not ? "!=" : "=", left, it);
      if (!first) emit(p, is_not ? OP_AND : OP_OR);
      first = 0;
    }
    return;
  }
  if (!left || !right)
  {
    fail(p, "malformed comparison, missing operand(s)");
    emit(p, OP_PUSH_TRUE);
    return;
  }
  compile_comparison(c, op, left, right);
}

int cqlops_program_build(const char* where, const CqlColumn* columns, const char* const* names, uint32_t column_count, CqlProgram* prog)
{
  memset(prog, 0, sizeof(*prog));
  Ctx c = { prog, columns, names, column_count };
  if (!where || !*where)
  {
    emit(prog, OP_PUSH_TRUE);
    emit(prog, OP_HALT);
    return 1;
  }
  Reader r = { where, 0, 0 };
  Node* root = read_node(&r);
  skip_ws(&r);
  if (r.failed || !root || r.s[r.i])
  {
    free_node(root);
    fail(prog, "malformed condition text");
    return 0;
  }
  compile(&c, root);
  free_node(root);
  emit(prog, OP_HALT);
  return prog->error[0] == 0;
}

/* qe_bytecode_program_max_stack_depth (query_exec.c:552-612) */
uint32_t cqlops_program_max_stack_depth(const CqlProgram* p)
{
  uint32_t depth = 0, max_depth = 0;
  uint64_t ip = 0;
  while (ip < p->word_count)
  {
    uint32_t op = p->words[ip++];
    switch (op)
    {
      case OP_PUSH_TRUE:
      case OP_PUSH_FALSE: depth += 1; break;
      case OP_LOAD_NUM_COL:
      case OP_PUSH_CONST:
        ip += 1;
        depth += 1;
        break;
      case OP_CMP_EQ: case OP_CMP_NE: case OP_CMP_LT: case OP_CMP_GT: case OP_CMP_LE: case OP_CMP_GE: case OP_AND: case OP_OR:
        depth -= 1;
        break;
      case OP_STR_EQ: case OP_STR_CONTAINS: case OP_TRIGRAM_SIM: case OP_EDIT_DISTANCE: case OP_STR_NE: case OP_STR_LT:
      case OP_STR_GT: case OP_STR_LE: case OP_STR_GE:
        ip += 3;
        depth += 1;
        break;
      default: ip = p->word_count; break;
    }
    if (depth > max_depth) max_depth = depth;
  }
  return max_depth;
}

/* The leaves of an AND-only tree of `column op number` comparisons on numeric columns, the shape
   scan_simple takes (qe_cpu_scan_collect_leaves + the checks of qe_scan_filter_selected :2526-2563).
   Returns the leaf count, 0 when the program has another shape. */
uint32_t cqlops_program_simple_leaves(const CqlProgram* p, CqlLeaf* out, uint32_t cap)
{
  uint32_t n = 0;
  uint64_t ip = 0;
  uint32_t pending = 0; /* comparisons not yet joined by AND */
  while (ip < p->word_count)
  {
    uint32_t op = p->words[ip++];
    if (op == OP_HALT) break;
    if (op == OP_LOAD_NUM_COL && ip + 3 <= p->word_count && p->words[ip + 1] == OP_PUSH_CONST)
    {
      uint32_t operand = p->words[ip];
      uint32_t k = p->words[ip + 2];
      uint32_t cmp = ip + 3 < p->word_count ? p->words[ip + 3] : 0;
      uint32_t simple = cmp == OP_CMP_EQ ? 0u : cmp == OP_CMP_LT ? 1u : cmp == OP_CMP_LE ? 2u : cmp == OP_CMP_GT ? 3u : cmp == OP_CMP_GE ? 4u : 99u;
      uint32_t type = (operand >> 8) & 0xffu, slot = operand & 0xffu;
      if (simple == 99u || n >= cap || !(type == CQLOPS_TYPE_U32 || type == CQLOPS_TYPE_I32 || type == CQLOPS_TYPE_F32 || type == CQLOPS_TYPE_F64))
        return 0;
      /* dictionary codes are U32 bindings of a string column: scan_simple keeps them out (:2546) */
      uint32_t b = 0;
      while (b < p->binding_count && p->binding_slot[b] != slot) b++;
      if (b == p->binding_count || p->binding_dict[b]) return 0;
      uint64_t bits = ((uint64_t)p->consts[k * 2 + 1] << 32) | p->consts[k * 2];
      double target;
      memcpy(&target, &bits, sizeof(target));
      out[n].column = p->binding_column[b];
      out[n].op = simple;
      out[n].target = target;
      n++;
      pending++;
      ip += 4;
      continue;
    }
    if (op == OP_AND && pending >= 2)
    {
      pending--;
      continue;
    }
    return 0;
  }
  return pending == 1 ? n : 0;
}

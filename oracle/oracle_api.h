/*
 * C interface shared by the two CPU oracles of the QuIDS rule step.
 *
 *   oracle/_ref/libquids_ref.so   the reference headers themselves (quids.hpp,
 *                                 rules/quantum_computer.hpp, rules/qcgd.hpp)
 *                                 compiled by oracle/Makefile from the
 *                                 reference source tree; x86 container only.
 *   oracle/_port/libquids_port.so oracle/quids_port.cpp, a restatement of the
 *                                 same algorithm written for this project; it
 *                                 builds anywhere (it is what runs on the GPU
 *                                 host as the CPU baseline and the parity
 *                                 oracle).
 *
 * This is TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py load these libraries, and
 * only as the checker or the timed CPU baseline -- never as the product path.
 *
 * Rule and modifier kinds use the same numbering as include/quids_gpu.h.
 * params layout (doubles):
 *   QUIDS_RULE_HADAMARD            [bit]
 *   QUIDS_RULE_QCGD_*              [theta, phi, xi]
 *   QUIDS_MOD_CNOT                 [control, target]
 *   QUIDS_MOD_X / _Y / _Z          [bit]
 *   QUIDS_MOD_QCGD_STEP / REVERSED []
 */
#ifndef QUIDS_ORACLE_API_H
#define QUIDS_ORACLE_API_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

void *qo_state_new(void);
void qo_state_free(void *st);
/* appends n objects (object i = objects[begin[i] .. begin[i]+size[i])), mag = 2n doubles */
int qo_state_load(void *st, uint64_t n, const uint8_t *objects, const uint64_t *begin,
                  const uint32_t *size, const double *mag);
uint64_t qo_state_num_object(void *st);
/* bytes of the packed store (object sizes padded to the current alignment) */
uint64_t qo_state_num_bytes(void *st);
/* writes the packed store: begin has n+1 entries, mag 2n doubles */
int qo_state_store(void *st, uint8_t *objects, uint64_t *begin, uint32_t *size, double *mag);
double qo_state_total_proba(void *st);

void qo_set_globals(double tolerance, int simple_truncation, uint32_t align_byte_length);
void qo_set_threads(int n);
int qo_get_threads(void);

/* one rule step: out <- rule(in); counters[0] = symbolic num_object,
 * counters[1] = num_object_after_interferences.  max_num_object = UINT64_MAX
 * means no truncation. */
int qo_simulate(void *in, int rule_kind, const double *params, void *out,
                uint64_t max_num_object, uint64_t *counters);
int qo_modifier(void *st, int modifier_kind, const double *params);

/* per-object rule callbacks, for rule-level parity tests */
uint64_t qo_hash_bytes(const uint8_t *b, uint64_t len);
uint64_t qo_qcgd_hash_graph(const uint8_t *b);
int qo_num_child(int rule_kind, const double *params, const uint8_t *obj, uint32_t size,
                 uint32_t *num_child, uint32_t *max_child_size);
/* mag: in = parent magnitude (2 doubles), out = child magnitude */
int qo_populate_child(int rule_kind, const double *params, const uint8_t *parent, uint32_t psize,
                      uint32_t child_id, uint8_t *child, uint32_t *csize, double *mag);
uint64_t qo_rule_hash(int rule_kind, const double *params, const uint8_t *obj, uint32_t size);

#ifdef __cplusplus
}
#endif
#endif

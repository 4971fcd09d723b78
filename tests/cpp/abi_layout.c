/* Prints sizeof / offsetof of the WFA2-lib structures a drop-in must match byte for byte:
 * wavefront_aligner_attr_t (every member, and every member of its alignment_system_t),
 * cigar_t, wavefront_align_status_t and the public members of wavefront_aligner_t.
 * Compiled twice by tests/test_abi_layout.py: against this library's include/wfa_gpu.h, and
 * (-DWITH_WFA2) against WFA2-lib's own headers; the two outputs must be identical. */
#include <stddef.h>
#include <stdio.h>

#ifdef WITH_WFA2
#include "wavefront/wavefront_align.h"
#else
#include "wfa_gpu.h"
#endif

#define SIZE(T) printf("sizeof %s %zu\n", #T, sizeof(T))
#define OFF(T, f) printf("offsetof %s.%s %zu\n", #T, #f, offsetof(T, f))

int main(void) {
  SIZE(wavefront_aligner_attr_t);
  OFF(wavefront_aligner_attr_t, distance_metric);
  OFF(wavefront_aligner_attr_t, alignment_scope);
  OFF(wavefront_aligner_attr_t, alignment_form);
  OFF(wavefront_aligner_attr_t, linear_penalties);
  OFF(wavefront_aligner_attr_t, affine_penalties);
  OFF(wavefront_aligner_attr_t, affine2p_penalties);
  OFF(wavefront_aligner_attr_t, heuristic);
  OFF(wavefront_aligner_attr_t, memory_mode);
  OFF(wavefront_aligner_attr_t, mm_allocator);
  OFF(wavefront_aligner_attr_t, plot);
  OFF(wavefront_aligner_attr_t, system);
  SIZE(alignment_form_t);
  OFF(alignment_form_t, span);
  OFF(alignment_form_t, extension);
  OFF(alignment_form_t, pattern_begin_free);
  OFF(alignment_form_t, text_end_free);
  SIZE(wavefront_heuristic_t);
  OFF(wavefront_heuristic_t, strategy);
  OFF(wavefront_heuristic_t, max_sw_score_k);
  SIZE(alignment_system_t);
  OFF(alignment_system_t, max_alignment_steps);
  OFF(alignment_system_t, probe_interval_global);
  OFF(alignment_system_t, probe_interval_compact);
  OFF(alignment_system_t, max_partial_compacts);
  OFF(alignment_system_t, max_memory_compact);
  OFF(alignment_system_t, max_memory_resident);
  OFF(alignment_system_t, max_memory_abort);
  OFF(alignment_system_t, verbose);
  OFF(alignment_system_t, check_alignment_correct);
  OFF(alignment_system_t, timer);
  OFF(alignment_system_t, max_num_threads);
  OFF(alignment_system_t, min_offsets_per_thread);
  SIZE(cigar_t);
  OFF(cigar_t, operations);
  OFF(cigar_t, max_operations);
  OFF(cigar_t, begin_offset);
  OFF(cigar_t, end_offset);
  OFF(cigar_t, score);
  OFF(cigar_t, end_v);
  OFF(cigar_t, end_h);
  OFF(cigar_t, has_misms);
  OFF(cigar_t, cigar_buffer);
  OFF(cigar_t, cigar_length);
  SIZE(wavefront_align_status_t);
  OFF(wavefront_align_status_t, status);
  OFF(wavefront_align_status_t, score);
  OFF(wavefront_align_status_t, dropped);
  OFF(wavefront_align_status_t, num_null_steps);
  OFF(wavefront_align_status_t, memory_used);
  SIZE(wavefront_aligner_t);
  OFF(wavefront_aligner_t, align_mode);
  OFF(wavefront_aligner_t, align_status);
  OFF(wavefront_aligner_t, alignment_scope);
  OFF(wavefront_aligner_t, alignment_form);
  OFF(wavefront_aligner_t, heuristic);
  OFF(wavefront_aligner_t, memory_mode);
  OFF(wavefront_aligner_t, component_begin);
  OFF(wavefront_aligner_t, component_end);
  OFF(wavefront_aligner_t, alignment_end_pos);
  OFF(wavefront_aligner_t, bialigner);
  OFF(wavefront_aligner_t, cigar);
  OFF(wavefront_aligner_t, mm_allocator);
  OFF(wavefront_aligner_t, system);
  return 0;
}

/* Prints sizeof/offsetof of the C ABI structs as JSON, so the test suite can check the Python ctypes
 * mirror (megamol_gb300/p2v.py) against the header the library was compiled with. */
#include <stddef.h>
#include <stdio.h>

#include "p2v.h"

#define F(T, m) printf("\"%s.%s\": %zu, ", #T, #m, offsetof(T, m))
#define S(T) printf("\"%s\": %zu, ", #T, sizeof(T))

int main(void) {
    printf("{");
    S(p2v_params); S(p2v_particle_list); S(p2v_frame); S(p2v_volume); S(p2v_stats);
    S(p2v_batch_item); S(p2v_tune_report); S(p2v_mmpld_info); S(p2v_mmpld_list_info); S(p2v_vector_grid_info);
    F(p2v_vector_grid_info, global_radius); F(p2v_vector_grid_info, col_max);
    F(p2v_particle_list, colour_type); F(p2v_particle_list, colour_data); F(p2v_particle_list, global_colour);
    F(p2v_mmpld_info, clipbox); F(p2v_mmpld_list_info, bbox); F(p2v_mmpld_list_info, clusters);
    F(p2v_params, sigma); F(p2v_params, kernel); F(p2v_params, ao_mode); F(p2v_params, aos_eval_fac);
    F(p2v_params, tile_z); F(p2v_params, batch_graph); F(p2v_params, vector_grid);
    F(p2v_params, aos_deposit); F(p2v_params, aos_clip_plane); F(p2v_params, ao_normals); F(p2v_params, test_hold_mma); F(p2v_params, slab_z1);
    F(p2v_params, batch_persistent); F(p2v_params, queue_wait_polls); F(p2v_params, test_hold_queue);
    F(p2v_params, sort_wait_polls); F(p2v_params, test_hold_sort); F(p2v_params, ao_march); F(p2v_params, ao_brick_order);
    F(p2v_batch_item, volume); F(p2v_batch_item, size);
    F(p2v_tune_report, ms_best); F(p2v_tune_report, cand_lanes); F(p2v_tune_report, cand_ms);
    F(p2v_tune_report, persistent); F(p2v_tune_report, cand_persistent);
    F(p2v_particle_list, count); F(p2v_particle_list, mem); F(p2v_particle_list, ao_out);
    F(p2v_frame, frame_id); F(p2v_frame, lists);
    F(p2v_volume, resolution); F(p2v_volume, min_value); F(p2v_volume, data_hash);
    F(p2v_stats, mass_sum); F(p2v_stats, ms_total); F(p2v_stats, ao_fallback); F(p2v_stats, cell_max_count); F(p2v_stats, ao_fetches);
    F(p2v_stats, ms_ao_kernel);
    printf("\"end\": 0}\n");
    return 0;
}

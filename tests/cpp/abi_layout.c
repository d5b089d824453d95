/* Prints sizeof / offsetof of the C ABI structs, for the ctypes layout test. */
#include <stddef.h>
#include <stdio.h>

#include "hd/hd.h"

#define F(T, m) printf("%s.%s %zu\n", #T, #m, offsetof(T, m))

int main(void) {
    printf("hd_result %zu\n", sizeof(hd_result));
    F(hd_result, sum_ab); F(hd_result, avg_hd); F(hd_result, status); F(hd_result, hd_robust);
    printf("hd_options %zu\n", sizeof(hd_options));
    F(hd_options, barrier_timeout_ns); F(hd_options, percentile); F(hd_options, tuning_table);
    F(hd_options, record_timings); F(hd_options, kernel); F(hd_options, steps_per_barrier); F(hd_options, label);
    printf("hd_timings %zu\n", sizeof(hd_timings));
    F(hd_timings, iterations); F(hd_timings, brick_z); F(hd_timings, brick_rows);
    printf("hd_pair_desc %zu\n", sizeof(hd_pair_desc));
    F(hd_pair_desc, W); F(hd_pair_desc, on_device);
    printf("hd_server_options %zu\n", sizeof(hd_server_options));
    F(hd_server_options, max_inflight); F(hd_server_options, metric);
    printf("hd_server_stats %zu\n", sizeof(hd_server_stats));
    F(hd_server_stats, bytes_peak);
    return 0;
}

/*
 * tracer_stats.cu: the Whitted kernel of tracer.cu compiled with per-thread
 * work counters (namespace qr_dev_stats, qr_launch_whitted_stats).  Only the
 * instrumented qr_render_stats call launches it; timed launches use the
 * counter-free build of tracer.cu.
 */
#define QR_STATS 1
#include "tracer.cu"

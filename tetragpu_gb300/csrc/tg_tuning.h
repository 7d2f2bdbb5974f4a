// tg_tuning.h -- tile parameters of the kernels, as chosen by the sweep in
// tetragpu_gb300/tune.py (python -m tetragpu_gb300.tune --apply rewrites the
// block below; tetragpu_gb300/tuning.json keeps the measurements).  A -D on
// the compiler's command line takes precedence (the sweep builds its
// candidates that way).
#pragma once
// BEGIN TUNED
#ifndef TG_STAR_WIN_B
#define TG_STAR_WIN_B 240
#endif
// END TUNED

// defaults of the rest
#ifndef TG_STAR_WIN
#define TG_STAR_WIN 256   // VT entries per window of star pass A
#endif
#ifndef TG_STAR_WIN_B
#define TG_STAR_WIN_B 224   // VT entries per window of star pass B
#endif
#ifndef TG_STAR_THREADS
#define TG_STAR_THREADS 256   // threads per star-pass block
#endif
#ifndef TG_STAR_HASH_BITS
#define TG_STAR_HASH_BITS 10   // log2 of pass A's (vertex, neighbour) table slots
#endif
#ifndef TG_EFA_LANES
#define TG_EFA_LANES 2   // lanes per owned edge for its EF count in pass A
#endif
#ifndef TG_VTS_THREADS
#define TG_VTS_THREADS 64   // threads per VT-sort block
#endif
#ifndef TG_EDGE_ITEMS
#define TG_EDGE_ITEMS 8   // edge slots per thread of the edge-offset pass
#endif
#ifndef TG_EDGE_MINB
#define TG_EDGE_MINB 8   // resident blocks per SM asked of the edge-offset pass
#endif
#ifndef TG_VTP_ROWS
#define TG_VTP_ROWS 8   // rows in flight per warp when copying VT into star order
#endif
#ifndef TG_VTP_MINB
#define TG_VTP_MINB 4   // resident blocks per SM asked of that copy
#endif
#ifndef TG_ADJ_WIN
#define TG_ADJ_WIN 256   // VV entries per window of the link adjacency
#endif
#ifndef TG_ADJ_THREADS
#define TG_ADJ_THREADS 128   // threads per link-adjacency block
#endif
#ifndef TG_EE_GROUP
#define TG_EE_GROUP 4   // lanes per edge for EE rows of at most 16 + 16 entries
#endif

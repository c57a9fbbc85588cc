/*
 * mg_plugin.cuh -- a new frontier algorithm on libmg's engine.
 *
 * The reference adds an algorithm by editing the hooks of
 * code/user_function.h:211-447 and rebuilding its binaries.  Here an
 * algorithm is an operator struct -- the static __device__ hooks and
 * capability flags described in mg_ops.cuh -- and
 *
 *     MG_FRONTIER_OPERATOR(name, Op)
 *
 * instantiates the hybrid push/pull frontier engine (the one mg_bfs, mg_sssp
 * and mg_bc run on) for it and defines
 *
 *     extern "C" mg_status name(mg_graph *g, int32_t source, const mg_opts *o,
 *                               int32_t *label_out, mg_run_info *info);
 *
 * with mg_bfs's conventions: source in the caller's vertex ids, labels (nv
 * int32, caller order) copied to label_out when it is non-NULL and kept on
 * the device for mg_result_device(g, MG_RES_LEVEL), mg_status codes,
 * options and run info as for the built-in algorithms.
 *
 * Build the operator's .cu file into its own shared library against this
 * one, for sm_103a:
 *     nvcc -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 -shared
 *          -Xcompiler -fPIC -I <repo>/include -I <repo>/multigraph_gb300/csrc
 *          op.cu -L <repo>/multigraph_gb300 -lmg -o libop.so
 * The engine's internals (multigraph_gb300/csrc) must come from the same
 * source tree libmg.so was built from.
 */
#ifndef MG_PLUGIN_CUH
#define MG_PLUGIN_CUH

#include "mg.h"
#include "mg_ops.cuh"
#include "mg_frontier_engine.cuh"

#define MG_FRONTIER_OPERATOR(NAME, OP)                                                                   \
    extern "C" mg_status NAME(mg_graph *g, int32_t source, const mg_opts *o, int32_t *label_out,         \
                              mg_run_info *info)                                                         \
    {                                                                                                    \
        return frontier_operator_run<OP>(g, source, o, label_out, info);                                 \
    }

#endif /* MG_PLUGIN_CUH */

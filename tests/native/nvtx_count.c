/* nvtx_count.c -- an NVTX injection library for the tests: loaded through
 * NVTX_INJECTION64_PATH, it takes over nvtxRangePushA and nvtxRangePop and
 * appends "push <name>" / "pop" lines to the file named by QEW_NVTX_LOG. Built
 * from the injection interface that the nvtx3 headers declare
 * (nvtxDetail/nvtxTypes.h: the callbacks export table and the core module's
 * function ids). */
#include <stdio.h>
#include <stdlib.h>

#include <nvtx3/nvToolsExt.h>

static FILE *g_log;

static int count_push(const char *message) {
    if (g_log) {
        fprintf(g_log, "push %s\n", message ? message : "");
        fflush(g_log);
    }
    return 0;
}

static int count_pop(void) {
    if (g_log) {
        fputs("pop\n", g_log);
        fflush(g_log);
    }
    return 0;
}

__attribute__((visibility("default"))) int InitializeInjectionNvtx2(
    NvtxGetExportTableFunc_t get_table) {
    const NvtxExportTableCallbacks *cb =
        (const NvtxExportTableCallbacks *)get_table(NVTX_ETID_CALLBACKS);
    NvtxFunctionTable table = 0;
    unsigned int size = 0;
    const char *path = getenv("QEW_NVTX_LOG");
    if (!cb || !path || !cb->GetModuleFunctionTable(NVTX_CB_MODULE_CORE, &table, &size) ||
        size <= NVTX_CBID_CORE_RangePop)
        return 0;
    g_log = fopen(path, "w");
    if (!g_log) return 0;
    *table[NVTX_CBID_CORE_RangePushA] = (NvtxFunctionPointer)count_push;
    *table[NVTX_CBID_CORE_RangePop] = (NvtxFunctionPointer)count_pop;
    return 1;
}

/* nvtx_recorder.c -- a minimal NVTX injection library for the tests.
 *
 * Loaded by the NVTX3 headers of the library under test when the environment
 * variable NVTX_INJECTION64_PATH names it: InitializeInjectionNvtx2 installs
 * handlers for range push (with attributes) and pop in the core callback
 * table, and every range is appended to the file named by
 * E2D_NVTX_RECORD as "push <name>" / "pop" lines. */
#include <stdio.h>
#include <stdlib.h>

#include <nvtx3/nvToolsExt.h>

static FILE* g_out;

static int record_push_ex(const nvtxEventAttributes_t* a) {
  if (g_out) {
    fprintf(g_out, "push %s\n", (a && a->messageType == NVTX_MESSAGE_TYPE_ASCII) ? a->message.ascii : "?");
    fflush(g_out);
  }
  return 0;
}

static int record_push_a(const char* msg) {
  if (g_out) {
    fprintf(g_out, "push %s\n", msg ? msg : "?");
    fflush(g_out);
  }
  return 0;
}

static int record_pop(void) {
  if (g_out) {
    fputs("pop\n", g_out);
    fflush(g_out);
  }
  return 0;
}

int InitializeInjectionNvtx2(NvtxGetExportTableFunc_t get_table) {
  const NvtxExportTableCallbacks* cb = (const NvtxExportTableCallbacks*)get_table(NVTX_ETID_CALLBACKS);
  NvtxFunctionTable table = 0;
  unsigned int size = 0;
  const char* path = getenv("E2D_NVTX_RECORD");
  if (!cb || !path || !cb->GetModuleFunctionTable(NVTX_CB_MODULE_CORE, &table, &size) || !table) return 0;
  if (size <= NVTX_CBID_CORE_RangePop) return 0;
  g_out = fopen(path, "a");
  if (!g_out) return 0;
  *table[NVTX_CBID_CORE_RangePushEx] = (NvtxFunctionPointer)record_push_ex;
  *table[NVTX_CBID_CORE_RangePushA] = (NvtxFunctionPointer)record_push_a;
  *table[NVTX_CBID_CORE_RangePop] = (NvtxFunctionPointer)record_pop;
  return 1;
}

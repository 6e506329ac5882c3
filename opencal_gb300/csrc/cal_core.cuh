/*
 * cal_core.cuh -- library-private engine shared by the 2D and 3D C APIs.
 *
 * One CalGrid per model holds:
 *   - the substates: per slot two device layers (SoA, cudaMalloc, 256-byte
 *     aligned) and two pinned host mirrors, with per-layer coherence flags;
 *   - the active-cell state on the device: byte flags, the compacted list of
 *     cells in the reference's order plus the same list as linear indices,
 *     and its length (an int in device memory, never read back per step);
 *   - the CUDA stream every operation of the model is queued on.
 *
 * Update semantics (OpenCAL-OMP/source/cal2D.c:758-776): rebuild the active
 * list, then copy next -> current for every registered substate, at the
 * active cells when the list is non-empty, else everywhere.  Without active
 * cells a substate that no process wrote since the last update already has
 * next == current everywhere, so its copy is skipped (device-side written
 * bits).  With active cells every registered substate is copied, because a
 * cell can re-enter the list with next != current.
 */
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "opencal/calCommon.h"

#define CAL_MAX_SUBSTATES_CORE 32
#define CAL_NTYPES 3
#define CAL_MAX_PROCESSES_CORE 32 /* CAL_MAX_ELEMENTARY_PROCESSES of cal2D.h */

namespace cal {

/* ---- error recording --------------------------------------------------- */
void set_error(CALError code, const std::string& msg);
bool cuda_ok(cudaError_t e, const char* what);

struct Layer {
    void* dev = nullptr;   /* device buffer */
    bool host_valid = true;
    bool dev_valid = true;
};

struct Sub {
    bool used = false;
    bool single = false;     /* single-layer: no next, not registered, not updated */
    int type = 0;            /* 0 byte, 1 int, 2 real */
    size_t elem = 1;
    Layer layer[2];          /* logical layers: 0 = current, 1 = next */
    void* host[2] = {nullptr, nullptr};
    bool next_stale = false; /* after a pointer swap next holds old data */
    bool forced_dirty = false;
    /* change tracking (2D models without active cells, CalGrid::tracking):
     *  trackable  false for good once a device pointer of the substate was
     *             handed out or its layers were swapped (writes the library
     *             does not see)
     *  track      the chg bitmap is exact: next == current outside its tiles
     *  uval_valid both layers hold `uval` (bit pattern) outside the tiles of
     *             the dev and chg bitmaps */
    bool trackable = true;
    bool track = true;
    bool uval_valid = true;
    unsigned long long uval = 0;
};

/* host-side bookkeeping that a step may change; restored when a graph
 * recording of the step is abandoned */
struct GridState {
    Sub sub[CAL_NTYPES][CAL_MAX_SUBSTATES_CORE];
    bool flags_host_valid, flags_dev_valid;
    int transfers;
    long swaps;
};

struct CalGrid {
    int dim = 2;
    int rows = 0, cols = 0, slices = 1;
    long long ncells = 0;
    int toroidal = 0;
    int active = 0; /* CAL_OPT_ACTIVE_CELLS */
    cudaStream_t stream = nullptr;

    Sub sub[CAL_NTYPES][CAL_MAX_SUBSTATES_CORE];
    void* pool[CAL_NTYPES] = {nullptr, nullptr, nullptr}; /* host handle pools */
    int nslot[CAL_NTYPES] = {0, 0, 0};

    /* active cells (device) */
    unsigned char* d_flags = nullptr;
    int* d_cells = nullptr;  /* dim ints per cell, reference order */
    int* d_lin = nullptr;    /* linear index per listed cell */
    int* d_count = nullptr;
    int* d_block_counts = nullptr; /* compaction scratch: ticket line + per-block counts */
    long long scratch_ints = 0;
    bool flags_host_valid = true, flags_dev_valid = true;
    unsigned char* h_flags = nullptr; /* host mirror (pinned) */
    /* 2D: a device word the process kernels set when they change a flag, so
     * that a compaction after a process that changed none keeps the list
     * (cal_core.cu, CompactGeom::dirty); flags written through the handed-out
     * device pointer are seen by the next explicit compaction
     * (calUpdateActiveCells2D) or after calMarkDeviceWritten2D, which set it */
    unsigned* d_flags_dirty = nullptr;
    unsigned* flags_dirty_word() const { return d_flags_dirty; }
    bool mark_flags_changed();

    unsigned* d_dirty = nullptr; /* [3] written-substate bits */
    /* change tracking: CAL_TILE_W x CAL_TILE_H tiles (include/opencal/
     * cal2DDevice.cuh), one bitmap of tile_words words per substate slot
     * (index type * CAL_MAX_SUBSTATES_CORE + slot) in d_chg (next may differ
     * from current) and d_dev (the layers may differ from the substate's
     * uniform value); d_untracked: [3] substates written by unsafe
     * operations since the last update, [3] the update kernel's ticket */
    bool tracking = false;
    /* bumped by every host-side event that invalidates tracked state (host
     * writes, one-layer fills, copies into both layers, handed-out device
     * pointers, swaps): a step recorded as a graph before such an event
     * holds decisions that no longer apply and is recorded again */
    long inval_epoch = 0;
    int tiles_x = 0, tiles_y = 0, tile_words = 0;
    unsigned* d_chg = nullptr;
    unsigned* d_dev = nullptr;
    unsigned* d_untracked = nullptr;
    /* tile skipping of pure processes: one must-run bitmap (tile_words
     * words) per process slot; the update and fill kernels set the bits of
     * the 3 x 3 tiles around every tile whose current layer they change, in
     * the first nrun bitmaps; run_epoch: inval_epoch when every bit was last
     * set (-1: never) */
    unsigned* d_run = nullptr;
    int nrun = 0;
    long run_epoch = -1;
    /* a skipping launch that deals its busy tiles over the blocks keeps the
     * bitmap unchanged while it runs: the tiles where the process changed
     * nothing are gathered in d_quiet (tile_words words, zero between
     * launches) and cleared from the bitmap by the launch's last block
     * (d_ticket counts the finished blocks, zero between launches) */
    unsigned* d_quiet = nullptr;
    unsigned* d_ticket = nullptr;
    int* d_step = nullptr;       /* step counter of a device-driven run */
    void* d_reduce_partial = nullptr; /* reduction scratch (per-block partials) */
    void* d_reduce_result = nullptr;  /* reduction result read back by the host */
    int transfers = 0;           /* host<->device coherence copies made so far */
    long swaps = 0;              /* pointer swaps made so far */
    int capturing = 0;
    bool written_since_update = true; /* a process kernel may have set written bits */

    /* lifecycle */
    bool init(int dim, int rows, int cols, int slices, int toroidal, int active);
    void destroy();

    /* substates */
    int add_sub(int type, bool single, void** cur_mirror, void** next_mirror);
    Sub& s(int type, int slot) { return sub[type][slot]; }

    /* coherence */
    bool to_device_all();                      /* every layer of every substate + flags */
    bool to_host(int type, int slot, int layer);
    bool load_from_host(int type, int slot, const void* src); /* caller's array -> both layers */
    bool store_to_host(int type, int slot, void* dst);        /* current layer -> caller's array */
    bool flags_to_host();
    void host_wrote(int type, int slot, int layer);
    void device_wrote_all();                   /* after a user process */
    bool repair_stale(int type, int slot);      /* next <- current after a swap */
    bool repair_all_stale();

    /* device operations */
    bool fill(int type, int slot, int layer, const void* value, bool at_active);
    bool fill_both(int type, int slot, const void* value); /* calInitSubstate: both layers, all (or active) cells */
    void untrack(int type, int slot);                    /* device pointer handed out: no tracking from now on */
    bool copy_next_to_current(const std::vector<std::pair<int, int>>& which, bool use_dirty, bool at_active);
    bool update_all();                         /* calUpdate: compaction + copies */
    bool compact();                            /* calUpdateActiveCells */
    bool clear_dirty();
    bool arm_runs();                           /* every tile must run again, for every process */
    bool swap(int type, int slot);
    bool sync();
    long long lin(int i, int j, int k) const
    {
        return dim == 2 ? (long long)i * cols + j : (long long)k * rows * cols + (long long)i * cols + j;
    }
    void launch_grid(int* gx, int* gy) const;
    void save(GridState* st) const;
    void restore(const GridState* st);
};

/* compaction of byte flags into the reference-ordered active list; scratch
 * holds compact_scratch_ints(cells) ints, the first of which (the ticket)
 * must be 0 before the first call: every call leaves it at 0 */
cudaError_t compact_flags(const unsigned char* flags, int dim, int rows, int cols, int slices, int* cells, int* lin,
                          int* count, int* scratch, long long scratch_ints, cudaStream_t stream,
                          unsigned* dirty = nullptr);
int compact_blocks_needed(long long ncells);
long long compact_scratch_ints(long long ncells);

} // namespace cal

// ci_plan.h -- host-side mesh preprocessing for the GB300 impact step.
//
// The element loop of the reference (include/dynamics_kernels.h:75-139) scatters each
// element's -f/m into the global acceleration in element order.  On the GPU that
// scatter becomes a deterministic two-level assembly without float atomics:
//
//  * elements are sorted along a 3D Hilbert curve of their centroids and cut into
//    contiguous CHUNKS; one CTA processes one chunk;
//  * every node is OWNED by the first chunk that touches it, and nodes are renumbered
//    so each chunk's owned nodes are contiguous: first its INTERIOR nodes (touched by
//    no other chunk), then its owned BOUNDARY nodes, each in first-touch order along
//    the curve; the other chunks touching a boundary node hold it as a GHOST;
//  * inside a chunk the elements are greedily coloured (no two elements of a colour
//    share a node) and sorted by colour, so the CTA adds element forces into its
//    shared-memory node accumulators colour by colour with plain read-modify-writes;
//  * each (chunk, local node) pair owns one SLOT; the chunk writes its partial node
//    sums to its slots and the node kernel sums a node's slots in chunk order.
//
// Every sum therefore has a fixed order and the result is bitwise reproducible.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace ci {

struct ChunkInfo {
  int elem_begin;   // first element (plan order)
  int elem_end;
  int own_begin;    // first owned node (plan order)
  int n_own;        // owned nodes are local ids [0, n_own)
  int n_local;      // owned + ghost
  int local_begin;  // offset of this chunk's entries in the local tables
  int n_int;        // interior nodes (touched by this chunk only) are local ids [0, n_int)
  int inst;         // instance of a batched solve (0 for a single mesh)
  int slot_begin;   // slot of interior node l is slot_begin + l (one slot each)
};

struct Plan {
  int N = 0, E = 0, npe = 0;
  int n_chunks = 0;
  int max_local = 0, max_colors = 0, max_chunk_elems = 0;
  long long n_ghosts = 0, n_boundary = 0;
  std::vector<ChunkInfo> chunks;
  std::vector<int> elem_orig;        // plan element -> original element
  std::vector<uint16_t> conn_local;  // [npe][E] local node ids, SoA by corner
  std::vector<uint8_t> color;        // [E]
  std::vector<int> node_orig;        // plan node -> original node
  std::vector<int> node_new;         // original node -> plan node
  std::vector<int> local_gid;        // [sum n_local] plan node id of each local node
  std::vector<int> local_slot;       // [sum n_local] slot of each (chunk, local node)
  std::vector<int> slot_row;         // [N+1] slots of node n: [slot_row[n], slot_row[n+1])
  std::vector<int> local_srow;       // [2 sum n_local] slot range of each local node's node
};

// Automatic chunking aims at this many chunks (CTAs) for small meshes: four per SM of a
// 152-SM GB300.  A constant, so a mesh's plan does not depend on the device.
constexpr int kDefaultTargetCtas = 608;

// Builds the plan.  chunk_elements / chunk_nodes <= 0 select defaults from the mesh
// size and target_ctas (<= 0: kDefaultTargetCtas).
bool build_plan(int N, int E, int npe, const double* xloc, const int* conn, int chunk_elements,
                int chunk_nodes, int target_ctas, Plan* plan, std::string* err);

// Dependency lists of the task kernel, CSR by chunk, each list sorted and unique:
// own[c] = the chunks owning one of chunk c's local nodes (its element tasks read their
// node records), touch[c] = the chunks holding a local entry of a node chunk c owns
// (its node tasks sum their partial forces).  Returns the longest list.
int flow_lists(const Plan& P, std::vector<int>* own_row, std::vector<int>* own_idx,
               std::vector<int>* touch_row, std::vector<int>* touch_idx);

// Task order of the chunks for the task kernel: reverse Cuthill-McKee on the graph of
// chunks sharing a node (the own lists, made symmetric), components in order of their
// lowest chunk, each from a pseudo-peripheral chunk, neighbours by degree then id.
// Chunks that share nodes get nearby positions, so every task's dependencies lie about
// one block of C tasks back in the claim order.
std::vector<int> flow_order(int C, const std::vector<int>& own_row, const std::vector<int>& own_idx);

// Host check of the plan invariants (used by tests through ci_plan_verify).
bool verify_plan(const Plan& p, const int* conn, std::string* err);

uint64_t hilbert_key3(uint32_t x, uint32_t y, uint32_t z, int bits);

}  // namespace ci

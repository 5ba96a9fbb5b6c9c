// legion.h -- a minimal, single-threaded stand-in for the early Legion
// high-level runtime API that LegionOrigins' apps/circuit/circuit.cc was
// written against (RegionRuntime::HighLevel, typed ptr_t<T>, templated
// PhysicalRegion<AT>).  The runtime shipped beside the app has moved on
// (LegionRuntime::, untyped pointers), so circuit.cc cannot be built as
// shipped.  This shim provides just enough of the old API to compile the
// reference's circuit.cc UNMODIFIED with -DUSING_SHARED and run its own
// main(), generator and CPU leaf tasks on one thread.
//
// TEST INFRASTRUCTURE ONLY: it exists to pin the oracle against the
// reference's own code.  Nothing in the product links it.
//
// Semantics reproduced (reference file:line):
//  * pointers are the reference's own ptr_t<T>/utptr_t from
//    runtime/common.h (compiled with TYPED_POINTERS), including their
//    ordering, which std::set in load_circuit relies on;
//  * PointerIterator enumerates a region's elements in ascending order,
//    as ElementMask::Enumerator does (runtime/shared_lowlevel.cc:1999-2030);
//  * reduce() on a read-write region applies REDOP::apply<true> in place;
//    on a reduction-only region it folds into a per-task instance
//    initialised to REDOP::identity (runtime/lowlevel.h:475-492); the
//    instances of an index launch are applied to the parent after the
//    launch, point by point in ascending order (one legal order of
//    runtime/shared_lowlevel.cc:2600-2760);
//  * index launches run their points one after another, in order.
//
// Hooks for the pinning harness (environment variables):
//  CKT_REFSHIM_DUMP=<prefix>      write every root region's bytes at unmap
//                                 (<prefix>.init.r<k>.bin) and at destroy
//                                 (<prefix>.final.r<k>.bin), k = creation order
//  CKT_REFSHIM_OVERRIDE=<prefix>  at the unmap that ends load_circuit,
//                                 replace root region k's bytes with
//                                 <prefix>.r<k>.bin when that file exists
#ifndef CKT_REFSHIM_LEGION_H
#define CKT_REFSHIM_LEGION_H

#include <cassert>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <vector>

template <typename T> struct ptr_t;
#include "common.h"  // the reference's runtime/common.h (TYPED_POINTERS)

enum LogLevel { LEVEL_SPEW, LEVEL_DEBUG, LEVEL_INFO, LEVEL_PRINT, LEVEL_WARNING, LEVEL_ERROR, LEVEL_NONE };

namespace RegionRuntime {

class Logger {
public:
  class Category {
  public:
    explicit Category(const char *name) : name_(name) {}
    void operator()(int level, const char *fmt, ...);
    void debug(const char *fmt, ...);
    void info(const char *fmt, ...);
    void warning(const char *fmt, ...);
  private:
    const char *name_;
  };
};

namespace LowLevel {
enum AccessorType { AccessorGeneric, AccessorArray, AccessorArrayReductionFold,
                    AccessorGPU, AccessorGPUReductionFold, AccessorReductionList };
template <AccessorType AT> class RegionInstanceAccessorUntyped {
public:
  void *array_base = nullptr;
};
struct DetailedTimer {
  static void clear_timers(void) {}
  static void report_timers(void) {}
};
}  // namespace LowLevel

namespace HighLevel {

using LowLevel::AccessorType;
using LowLevel::AccessorGeneric;

typedef unsigned TaskID;
typedef unsigned PartitionID;
typedef unsigned ProjectionID;
typedef unsigned ReductionOpID;
typedef unsigned RegionID;

enum PrivilegeMode { NO_ACCESS, READ_ONLY, READ_WRITE, REDUCE };
enum AllocateMode { NO_MEMORY, ALLOCABLE, FREEABLE };
enum CoherenceProperty { EXCLUSIVE, ATOMIC, SIMULTANEOUS, RELAXED };

struct Processor {
  enum Kind { TOC_PROC, LOC_PROC, UTIL_PROC };
  unsigned id;
  static const Processor NO_PROC;
  bool operator<(const Processor &o) const { return id < o.id; }
  bool operator==(const Processor &o) const { return id == o.id; }
  bool operator!=(const Processor &o) const { return id != o.id; }
};

struct Memory {
  unsigned id;
  static const Memory NO_MEMORY;
  bool operator<(const Memory &o) const { return id < o.id; }
  bool operator==(const Memory &o) const { return id == o.id; }
  bool operator!=(const Memory &o) const { return id != o.id; }
};

struct ProcessorMemoryAffinity {
  Processor p;
  Memory m;
  unsigned bandwidth;
  unsigned latency;
};

class Machine {
public:
  Machine(void);
  const std::set<Processor> &get_all_processors(void) const { return procs_; }
  Processor::Kind get_processor_kind(Processor p) const;
  int get_proc_mem_affinity(std::vector<ProcessorMemoryAffinity> &result,
                            Processor restrict_proc = Processor::NO_PROC,
                            Memory restrict_mem = Memory::NO_MEMORY);
private:
  std::set<Processor> procs_;
  std::vector<Memory> mems_;
};

struct LogicalRegion {
  RegionID id;
  bool operator==(const LogicalRegion &o) const { return id == o.id; }
  bool operator<(const LogicalRegion &o) const { return id < o.id; }
};

struct Partition {
  PartitionID id;
};

class IndexPoint : public std::vector<int> {
public:
  IndexPoint(void) {}
  explicit IndexPoint(int dim) : std::vector<int>((size_t)dim, 0) {}
};

struct Range {
  int start, stop, stride;
  Range(void) : start(0), stop(-1), stride(1) {}
  Range(int a, int b, int s = 1) : start(a), stop(b), stride(s) {}
};

struct RangeSplit {
  std::vector<Range> ranges;
  Processor proc;
  bool recurse;
};

class TaskArgument {
public:
  TaskArgument(void) {}
  TaskArgument(const void *arg, size_t size)
      : bytes_((const char *)arg, (const char *)arg + (arg ? size : 0)) {}
  const void *get_ptr(void) const { return bytes_.empty() ? nullptr : bytes_.data(); }
  size_t get_size(void) const { return bytes_.size(); }
private:
  std::vector<char> bytes_;
};

class ArgumentMap {
public:
  TaskArgument &operator[](const IndexPoint &p) { return args_[p]; }
  const TaskArgument *find(const IndexPoint &p) const {
    auto it = args_.find(p);
    return it == args_.end() ? nullptr : &it->second;
  }
private:
  std::map<IndexPoint, TaskArgument> args_;
};

class FutureMap {
public:
  void wait_all_results(void) {}
  void release(void) {}
};

struct InputArgs {
  char **argv;
  int argc;
};

struct RegionRequirement {
  enum HandleKind { REGION_HANDLE, PARTITION_HANDLE };
  HandleKind kind;
  LogicalRegion region;
  PartitionID partition;
  ProjectionID projection;
  PrivilegeMode privilege;
  ReductionOpID redop;
  AllocateMode alloc;
  CoherenceProperty prop;
  LogicalRegion parent;

  RegionRequirement(void) {}
  RegionRequirement(LogicalRegion r, PrivilegeMode priv, AllocateMode a,
                    CoherenceProperty c, LogicalRegion par)
      : kind(REGION_HANDLE), region(r), partition(0), projection(0), privilege(priv),
        redop(0), alloc(a), prop(c), parent(par) {}
  RegionRequirement(PartitionID pid, ProjectionID proj, PrivilegeMode priv,
                    AllocateMode a, CoherenceProperty c, LogicalRegion par)
      : kind(PARTITION_HANDLE), region(), partition(pid), projection(proj),
        privilege(priv), redop(0), alloc(a), prop(c), parent(par) {}
  RegionRequirement(Partition p, ProjectionID proj, PrivilegeMode priv,
                    AllocateMode a, CoherenceProperty c, LogicalRegion par)
      : RegionRequirement(p.id, proj, priv, a, c, par) {}
  RegionRequirement(PartitionID pid, ProjectionID proj, ReductionOpID op,
                    AllocateMode a, CoherenceProperty c, LogicalRegion par)
      : kind(PARTITION_HANDLE), region(), partition(pid), projection(proj),
        privilege(REDUCE), redop(op), alloc(a), prop(c), parent(par) {}
};

// ---------------------------------------------------------------------------
// Region storage: every root region owns one byte array; subregions are
// ascending element lists over their root's storage.
// ---------------------------------------------------------------------------
struct RegionData {
  RegionID root;                  // root region id (self for roots)
  size_t elem_size;
  std::vector<char> *storage;     // root's storage
  unsigned *allocated;            // root's allocated count
  std::vector<unsigned> elems;    // ascending (subregions only)
  bool is_root;
};

class PointerIterator {
public:
  explicit PointerIterator(std::vector<unsigned> elems) : elems_(std::move(elems)), pos_(0) {}
  bool has_next(void) const { return pos_ < elems_.size(); }
  template <typename T> ptr_t<T> next(void) {
    ptr_t<T> p;
    p.value = elems_[pos_++];
    return p;
  }
private:
  std::vector<unsigned> elems_;
  size_t pos_;
};

struct RedopInfo {
  size_t sizeof_rhs;
  void (*init)(void *rhs);
  void (*apply)(void *lhs, const void *rhs);
};

struct PhysicalState {
  RegionData *data;        // the logical region this instance is of
  bool reduction_only;
  ReductionOpID redop;
  std::vector<char> fold;  // reduction-only instance, indexed by absolute ptr
};

template <AccessorType AT> class PhysicalRegion {
public:
  PhysicalRegion(void) : st_(nullptr) {}
  explicit PhysicalRegion(PhysicalState *st) : st_(st) {}

  template <typename T> T read(ptr_t<T> ptr) const {
    assert(!st_->reduction_only);
    T val;
    std::memcpy(&val, st_->data->storage->data() + (size_t)ptr.value * st_->data->elem_size,
                sizeof(T));
    return val;
  }
  template <typename T> void write(ptr_t<T> ptr, const T &val) const {
    assert(!st_->reduction_only);
    std::memcpy(st_->data->storage->data() + (size_t)ptr.value * st_->data->elem_size, &val,
                sizeof(T));
  }
  template <typename T, typename REDOP, typename RHS> void reduce(ptr_t<T> ptr, RHS newval) const {
    if (st_->reduction_only) {
      RHS val;
      std::memcpy(&val, st_->fold.data() + (size_t)ptr.value * sizeof(RHS), sizeof(RHS));
      REDOP::template fold<true>(val, newval);
      std::memcpy(st_->fold.data() + (size_t)ptr.value * sizeof(RHS), &val, sizeof(RHS));
    } else {
      T val = read(ptr);
      REDOP::template apply<true>(val, newval);
      write(ptr, val);
    }
  }
  PointerIterator *iterator(void) const;
  void wait_until_valid(void) const {}
  template <typename T> ptr_t<T> alloc(unsigned count = 1) const {
    ptr_t<T> first;
    first.value = *st_->data->allocated;
    *st_->data->allocated += count;
    assert((size_t)*st_->data->allocated * st_->data->elem_size <= st_->data->storage->size());
    return first;
  }
  PhysicalState *state(void) const { return st_; }
private:
  PhysicalState *st_;
};

struct ContextImpl;
typedef ContextImpl *Context;

class HighLevelRuntime;
class Mapper;

struct Task {
  TaskID task_id;
  bool is_index_space;
  IndexPoint point;
  const IndexPoint &get_index_point(void) const { return point; }
};

class Mapper {
public:
  Mapper(Machine *m, HighLevelRuntime *rt, Processor local);
  virtual ~Mapper(void) {}
protected:
  void decompose_range_space(unsigned cur_depth, unsigned max_depth,
                             const std::vector<Range> &index_space,
                             std::vector<Range> &chunk, std::vector<RangeSplit> &chunks,
                             unsigned &proc_index, std::vector<Processor> &targets);
  Machine *machine;
  HighLevelRuntime *runtime;
  Processor local_proc;
  Processor::Kind proc_kind;
  std::vector<Memory> memory_stack;
  std::vector<Processor> proc_group;
};

typedef void (*SingleTaskFn)(const void *, size_t,
                             std::vector<PhysicalRegion<AccessorGeneric> > &, Context,
                             HighLevelRuntime *);
typedef void (*IndexTaskFn)(const void *, size_t, const void *, size_t, const IndexPoint &,
                            std::vector<PhysicalRegion<AccessorGeneric> > &, Context,
                            HighLevelRuntime *);
typedef void (*RegistrationCallbackFn)(Machine *, HighLevelRuntime *, Processor);

class HighLevelRuntime {
public:
  static void set_registration_callback(RegistrationCallbackFn fn);
  static void set_top_level_task_id(TaskID id);
  template <SingleTaskFn FN>
  static TaskID register_single_task(TaskID id, Processor::Kind kind, const char *name) {
    if (kind == Processor::LOC_PROC) single_tasks()[id] = FN;
    (void)name;
    return id;
  }
  template <IndexTaskFn FN>
  static TaskID register_index_task(TaskID id, Processor::Kind kind, const char *name) {
    if (kind == Processor::LOC_PROC) index_tasks()[id] = FN;
    (void)name;
    return id;
  }
  template <typename REDOP> static void register_reduction_op(ReductionOpID id) {
    RedopInfo info;
    info.sizeof_rhs = sizeof(typename REDOP::RHS);
    info.init = [](void *rhs) {
      typename REDOP::RHS v = REDOP::identity;
      std::memcpy(rhs, &v, sizeof(v));
    };
    info.apply = [](void *lhs, const void *rhs) {
      typename REDOP::LHS l;
      typename REDOP::RHS r;
      std::memcpy(&l, lhs, sizeof(l));
      std::memcpy(&r, rhs, sizeof(r));
      REDOP::template apply<true>(l, r);
      std::memcpy(lhs, &l, sizeof(l));
    };
    redops()[id] = info;
  }
  static int start(int argc, char **argv);

  void replace_default_mapper(Mapper *m);
  LogicalRegion create_logical_region(Context ctx, size_t elem_size, unsigned num_elmts);
  void destroy_logical_region(Context ctx, LogicalRegion handle);
  template <AccessorType AT>
  PhysicalRegion<AT> map_region(Context ctx, const RegionRequirement &req) {
    return PhysicalRegion<AT>(make_physical(req.region, req));
  }
  template <AccessorType AT> void unmap_region(Context ctx, PhysicalRegion<AT> &region) {
    unmap_state(region.state());
  }
  Partition create_partition(Context ctx, LogicalRegion parent,
                             const std::vector<std::set<utptr_t> > &coloring,
                             bool disjoint = true);
  LogicalRegion get_subregion(Context ctx, Partition part, unsigned color);
  FutureMap execute_index_space(Context ctx, TaskID task_id,
                                const std::vector<Range> &index_space,
                                const std::vector<RegionRequirement> &regions,
                                const TaskArgument &global_arg, const ArgumentMap &arg_map,
                                bool must);

  RegionData *region_data(RegionID id) { return regions_.at(id); }

private:
  static std::map<TaskID, SingleTaskFn> &single_tasks(void);
  static std::map<TaskID, IndexTaskFn> &index_tasks(void);
  static std::map<ReductionOpID, RedopInfo> &redops(void);
  PhysicalState *make_physical(LogicalRegion r, const RegionRequirement &req);
  void unmap_state(PhysicalState *st);
  void dump_root(RegionID id, const char *stage);

  std::map<RegionID, RegionData *> regions_;
  std::vector<RegionID> roots_;
  std::map<PartitionID, std::vector<RegionID> > partitions_;
  std::vector<PhysicalState *> states_;
  std::vector<Mapper *> mappers_;
  RegionID next_region_ = 1;
  PartitionID next_partition_ = 1;
  int unmaps_ = 0;
};

template <AccessorType AT> PointerIterator *PhysicalRegion<AT>::iterator(void) const {
  if (st_->data->is_root) {
    std::vector<unsigned> all(*st_->data->allocated);
    for (unsigned i = 0; i < all.size(); i++) all[i] = i;
    return new PointerIterator(std::move(all));
  }
  return new PointerIterator(st_->data->elems);
}

}  // namespace HighLevel
}  // namespace RegionRuntime

#endif

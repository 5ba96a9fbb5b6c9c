// refshim.cc -- implementation of the single-threaded Legion-API stand-in in
// legion.h.  TEST INFRASTRUCTURE ONLY (pins the oracle against the
// reference's own apps/circuit/circuit.cc).
#include "legion.h"

#include <algorithm>
#include <cstdarg>
#include <string>

namespace RegionRuntime {

static bool verbose(void) { return std::getenv("CKT_REFSHIM_VERBOSE") != nullptr; }

void Logger::Category::operator()(int level, const char *fmt, ...) {
  if (!verbose()) return;
  va_list ap;
  va_start(ap, fmt);
  std::fprintf(stderr, "[%s:%d] ", name_, level);
  std::vfprintf(stderr, fmt, ap);
  std::fprintf(stderr, "\n");
  va_end(ap);
}
#define CKT_LOG_FN(NAME)                                   \
  void Logger::Category::NAME(const char *fmt, ...) {      \
    if (!verbose()) return;                                \
    va_list ap;                                            \
    va_start(ap, fmt);                                     \
    std::fprintf(stderr, "[%s] ", name_);                  \
    std::vfprintf(stderr, fmt, ap);                        \
    std::fprintf(stderr, "\n");                            \
    va_end(ap);                                            \
  }
CKT_LOG_FN(debug)
CKT_LOG_FN(info)
CKT_LOG_FN(warning)

namespace HighLevel {

const Processor Processor::NO_PROC = {0};
const Memory Memory::NO_MEMORY = {0};

Machine::Machine(void) {
  procs_.insert(Processor{1});
  mems_.push_back(Memory{1});
  mems_.push_back(Memory{2});
}

Processor::Kind Machine::get_processor_kind(Processor p) const {
  (void)p;
  return Processor::LOC_PROC;
}

int Machine::get_proc_mem_affinity(std::vector<ProcessorMemoryAffinity> &result,
                                   Processor restrict_proc, Memory restrict_mem) {
  for (const Processor &p : procs_) {
    if (restrict_proc != Processor::NO_PROC && p != restrict_proc) continue;
    for (const Memory &m : mems_) {
      if (restrict_mem != Memory::NO_MEMORY && m != restrict_mem) continue;
      result.push_back(ProcessorMemoryAffinity{p, m, 100, 1});
    }
  }
  return (int)result.size();
}

Mapper::Mapper(Machine *m, HighLevelRuntime *rt, Processor local)
    : machine(m), runtime(rt), local_proc(local), proc_kind(Processor::LOC_PROC) {
  memory_stack.push_back(Memory{1});
  memory_stack.push_back(Memory{2});
  proc_group.push_back(local);
}

void Mapper::decompose_range_space(unsigned, unsigned, const std::vector<Range> &index_space,
                                   std::vector<Range> &, std::vector<RangeSplit> &chunks,
                                   unsigned &, std::vector<Processor> &targets) {
  RangeSplit s;
  s.ranges = index_space;
  s.proc = targets.empty() ? local_proc : targets.front();
  s.recurse = false;
  chunks.push_back(s);
}

static RegistrationCallbackFn g_reg_cb = nullptr;
static TaskID g_top_id = 0;

std::map<TaskID, SingleTaskFn> &HighLevelRuntime::single_tasks(void) {
  static std::map<TaskID, SingleTaskFn> m;
  return m;
}
std::map<TaskID, IndexTaskFn> &HighLevelRuntime::index_tasks(void) {
  static std::map<TaskID, IndexTaskFn> m;
  return m;
}
std::map<ReductionOpID, RedopInfo> &HighLevelRuntime::redops(void) {
  static std::map<ReductionOpID, RedopInfo> m;
  return m;
}

void HighLevelRuntime::set_registration_callback(RegistrationCallbackFn fn) { g_reg_cb = fn; }
void HighLevelRuntime::set_top_level_task_id(TaskID id) { g_top_id = id; }

int HighLevelRuntime::start(int argc, char **argv) {
  HighLevelRuntime *rt = new HighLevelRuntime();
  Machine *machine = new Machine();
  Processor local = {1};
  if (g_reg_cb) g_reg_cb(machine, rt, local);
  InputArgs in;
  in.argv = argv;
  in.argc = argc;
  std::vector<PhysicalRegion<AccessorGeneric> > none;
  auto it = single_tasks().find(g_top_id);
  if (it == single_tasks().end()) {
    std::fprintf(stderr, "refshim: no top-level task\n");
    return 1;
  }
  it->second(&in, sizeof(in), none, nullptr, rt);
  return 0;
}

void HighLevelRuntime::replace_default_mapper(Mapper *m) { mappers_.push_back(m); }

LogicalRegion HighLevelRuntime::create_logical_region(Context, size_t elem_size,
                                                      unsigned num_elmts) {
  RegionData *d = new RegionData();
  const RegionID id = next_region_++;
  d->root = id;
  d->elem_size = elem_size;
  d->storage = new std::vector<char>(elem_size * (size_t)num_elmts, 0);
  d->allocated = new unsigned(0);
  d->is_root = true;
  regions_[id] = d;
  roots_.push_back(id);
  return LogicalRegion{id};
}

void HighLevelRuntime::dump_root(RegionID id, const char *stage) {
  const char *prefix = std::getenv("CKT_REFSHIM_DUMP");
  if (!prefix) return;
  size_t k = 0;
  while (k < roots_.size() && roots_[k] != id) k++;
  const std::string path = std::string(prefix) + "." + stage + ".r" + std::to_string(k) + ".bin";
  RegionData *d = regions_.at(id);
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) return;
  std::fwrite(d->storage->data(), 1, (size_t)*d->allocated * d->elem_size, f);
  std::fclose(f);
}

void HighLevelRuntime::destroy_logical_region(Context, LogicalRegion handle) {
  RegionData *d = regions_.at(handle.id);
  if (d->is_root) dump_root(handle.id, "final");
}

PhysicalState *HighLevelRuntime::make_physical(LogicalRegion r, const RegionRequirement &req) {
  PhysicalState *st = new PhysicalState();
  st->data = regions_.at(r.id);
  st->reduction_only = (req.privilege == REDUCE);
  st->redop = req.redop;
  if (st->reduction_only) {
    const RedopInfo &info = redops().at(req.redop);
    const size_t n = st->data->storage->size() / st->data->elem_size;
    st->fold.assign(n * info.sizeof_rhs, 0);
    for (size_t i = 0; i < n; i++) info.init(st->fold.data() + i * info.sizeof_rhs);
  }
  states_.push_back(st);
  return st;
}

void HighLevelRuntime::unmap_state(PhysicalState *st) {
  RegionData *d = st->data;
  if (!d->is_root) return;
  dump_root(d->root, "init");
  const char *prefix = std::getenv("CKT_REFSHIM_OVERRIDE");
  if (!prefix) return;
  size_t k = 0;
  while (k < roots_.size() && roots_[k] != d->root) k++;
  const std::string path = std::string(prefix) + ".r" + std::to_string(k) + ".bin";
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return;
  const size_t want = (size_t)*d->allocated * d->elem_size;
  const size_t got = std::fread(d->storage->data(), 1, want, f);
  std::fclose(f);
  if (got != want) {
    std::fprintf(stderr, "refshim: override %s has %zu bytes, expected %zu\n", path.c_str(), got,
                 want);
    std::exit(2);
  }
}

Partition HighLevelRuntime::create_partition(Context, LogicalRegion parent,
                                             const std::vector<std::set<utptr_t> > &coloring,
                                             bool) {
  RegionData *p = regions_.at(parent.id);
  const PartitionID pid = next_partition_++;
  std::vector<RegionID> subs;
  for (const std::set<utptr_t> &color : coloring) {
    RegionData *d = new RegionData();
    const RegionID id = next_region_++;
    d->root = p->root;
    d->elem_size = p->elem_size;
    d->storage = p->storage;
    d->allocated = p->allocated;
    d->is_root = false;
    for (const utptr_t &u : color) d->elems.push_back(u.value);
    std::sort(d->elems.begin(), d->elems.end());
    regions_[id] = d;
    subs.push_back(id);
  }
  partitions_[pid] = subs;
  return Partition{pid};
}

LogicalRegion HighLevelRuntime::get_subregion(Context, Partition part, unsigned color) {
  return LogicalRegion{partitions_.at(part.id).at(color)};
}

FutureMap HighLevelRuntime::execute_index_space(Context ctx, TaskID task_id,
                                                const std::vector<Range> &index_space,
                                                const std::vector<RegionRequirement> &regions,
                                                const TaskArgument &global_arg,
                                                const ArgumentMap &arg_map, bool) {
  auto it = index_tasks().find(task_id);
  if (it == index_tasks().end()) {
    std::fprintf(stderr, "refshim: task %u has no CPU variant\n", task_id);
    std::exit(2);
  }
  std::vector<PhysicalState *> pending;  // reduction instances, point order
  for (const Range &r : index_space) {
    for (int p = r.start; p <= r.stop; p += r.stride) {
      IndexPoint pt(1);
      pt[0] = p;
      std::vector<PhysicalRegion<AccessorGeneric> > regs;
      for (const RegionRequirement &req : regions) {
        LogicalRegion lr = req.kind == RegionRequirement::PARTITION_HANDLE
                               ? LogicalRegion{partitions_.at(req.partition).at((size_t)p)}
                               : req.region;
        PhysicalState *st = make_physical(lr, req);
        if (st->reduction_only) pending.push_back(st);
        regs.push_back(PhysicalRegion<AccessorGeneric>(st));
      }
      const TaskArgument *local = arg_map.find(pt);
      it->second(global_arg.get_ptr(), global_arg.get_size(),
                 local ? local->get_ptr() : nullptr, local ? local->get_size() : 0, pt, regs,
                 ctx, this);
    }
  }
  // Apply every reduction instance to its parent, point by point.
  for (PhysicalState *st : pending) {
    const RedopInfo &info = redops().at(st->redop);
    RegionData *d = st->data;
    for (unsigned e : d->elems)
      info.apply(d->storage->data() + (size_t)e * d->elem_size,
                 st->fold.data() + (size_t)e * info.sizeof_rhs);
  }
  return FutureMap();
}

}  // namespace HighLevel
}  // namespace RegionRuntime

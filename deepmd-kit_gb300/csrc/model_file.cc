// Reader of frozen DeePMD-kit PyTorch model files (.pth) for se_e2_a energy
// models, without libtorch.
//
// A .pth written by `dp --pt freeze` (torch.jit.save of the scripted
// EnergyModel, deepmd/pt/entrypoints/main.py freeze) is a zip archive:
//   <name>/data.pkl      the module tree as a pickle (protocol 2): modules are
//                        objects whose state dict holds their attributes,
//                        submodules, parameters and buffers; tensors are
//                        torch._utils._rebuild_tensor_v2(storage, offset,
//                        size, stride, ...) with the storage a persistent id
//                        ('storage', <type>, <key>, <location>, <numel>);
//   <name>/data/<key>    the raw little-endian bytes of storage <key>;
//   <name>/code/...      TorchScript source (not needed here).
// The model configuration is the JSON string attribute `model_def_script` of
// the root module (the "model" section of the training input).  Weights are
// read by their state-dict names (deepmd/pt/model/descriptor/se_a.py:534-576,
// deepmd/pt/model/task/fitting.py, deepmd/pt/model/atomic_model).
//
// Only what this reader needs of each format is implemented: stored (not
// deflated) zip entries, with or without zip64 records; the pickle opcodes
// torch.jit.save emits; JSON without \u escapes beyond ASCII.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "dpgb.h"

namespace dpgb {
void set_error(const std::string& msg);
void clear_error();
}  // namespace dpgb

namespace {

using dpgb::set_error;

struct Fail {
  std::string msg;
};
[[noreturn]] void fail(const std::string& m) { throw Fail{m}; }

// ---------------------------------------------------------------- zip ---
uint64_t rd_le(const std::string& b, size_t at, int n) {
  if (at + n > b.size()) fail("zip: truncated archive");
  uint64_t v = 0;
  for (int i = n - 1; i >= 0; --i) v = (v << 8) | (unsigned char)b[at + i];
  return v;
}

struct ZipEntry {
  size_t data = 0, size = 0;
  int method = 0;
};

std::map<std::string, ZipEntry> zip_index(const std::string& b) {
  // end of central directory: the last "PK\5\6" within the trailing 64 KiB
  if (b.size() < 22) fail("zip: not an archive");
  size_t eocd = std::string::npos;
  for (size_t i = b.size() - 22 + 1; i-- > 0 && b.size() - i <= 65557;)
    if (rd_le(b, i, 4) == 0x06054b50u) {
      eocd = i;
      break;
    }
  if (eocd == std::string::npos) fail("zip: no end-of-central-directory record");
  uint64_t n_ent = rd_le(b, eocd + 10, 2), cd_off = rd_le(b, eocd + 16, 4);
  if (n_ent == 0xFFFF || cd_off == 0xFFFFFFFFu) {  // zip64: locator just before the record
    if (eocd < 20 || rd_le(b, eocd - 20, 4) != 0x07064b50u) fail("zip: zip64 locator missing");
    const uint64_t rec = rd_le(b, eocd - 20 + 8, 8);
    if (rd_le(b, rec, 4) != 0x06064b50u) fail("zip: bad zip64 record");
    n_ent = rd_le(b, rec + 32, 8);
    cd_off = rd_le(b, rec + 48, 8);
  }
  std::map<std::string, ZipEntry> out;
  size_t p = cd_off;
  for (uint64_t e = 0; e < n_ent; ++e) {
    if (rd_le(b, p, 4) != 0x02014b50u) fail("zip: bad central directory entry");
    const int method = (int)rd_le(b, p + 10, 2);
    uint64_t csize = rd_le(b, p + 20, 4), usize = rd_le(b, p + 24, 4);
    const size_t nlen = rd_le(b, p + 28, 2), xlen = rd_le(b, p + 30, 2), clen = rd_le(b, p + 32, 2);
    uint64_t loff = rd_le(b, p + 42, 4);
    const std::string name = b.substr(p + 46, nlen);
    // zip64 extended information: the fields stored as 0xFFFFFFFF, in order
    for (size_t x = p + 46 + nlen; x + 4 <= p + 46 + nlen + xlen;) {
      const uint64_t id = rd_le(b, x, 2), sz = rd_le(b, x + 2, 2);
      if (id == 0x0001) {
        size_t q = x + 4;
        if (usize == 0xFFFFFFFFu) usize = rd_le(b, q, 8), q += 8;
        if (csize == 0xFFFFFFFFu) csize = rd_le(b, q, 8), q += 8;
        if (loff == 0xFFFFFFFFu) loff = rd_le(b, q, 8), q += 8;
      }
      x += 4 + sz;
    }
    if (rd_le(b, loff, 4) != 0x04034b50u) fail("zip: bad local header of " + name);
    ZipEntry z;
    z.data = loff + 30 + rd_le(b, loff + 26, 2) + rd_le(b, loff + 28, 2);
    z.size = csize;
    z.method = method;
    if (z.data + z.size > b.size()) fail("zip: entry past the end: " + name);
    (void)usize;
    out[name] = z;
    p += 46 + nlen + xlen + clen;
  }
  return out;
}

// ------------------------------------------------------------- pickle ---
struct PV;
using P = std::shared_ptr<PV>;
struct PV {
  enum Kind { None, Bool, Int, Float, Str, Tuple, List, Dict, Global, Object, Tensor, Storage, Mark } k = None;
  bool b = false;
  long long i = 0;
  double f = 0.0;
  std::string s;                         // Str; Global "module name"; Storage type
  std::vector<P> items;                  // Tuple, List
  std::vector<std::pair<P, P>> dict;     // Dict (insertion order)
  P cls, state;                          // Object
  // Tensor: storage, offset, sizes, strides; Storage: key, numel (s = type)
  P storage;
  long long offset = 0, numel = 0;
  std::vector<long long> size, stride;
  std::string key;
};

P mk(PV::Kind k) {
  auto p = std::make_shared<PV>();
  p->k = k;
  return p;
}

long long as_int(const P& p) {
  if (!p || (p->k != PV::Int && p->k != PV::Bool)) fail("pickle: integer expected");
  return p->k == PV::Bool ? (long long)p->b : p->i;
}

std::vector<long long> int_tuple(const P& p) {
  if (!p || (p->k != PV::Tuple && p->k != PV::List)) fail("pickle: tuple of integers expected");
  std::vector<long long> v;
  for (auto& x : p->items) v.push_back(as_int(x));
  return v;
}

P unpickle(const std::string& d) {
  std::vector<P> st;
  std::vector<size_t> marks;
  std::map<long long, P> memo;
  size_t pc = 0;
  auto rd = [&](int n) {
    const uint64_t v = rd_le(d, pc, n);
    pc += n;
    return v;
  };
  auto pop = [&]() {
    if (st.empty()) fail("pickle: stack underflow");
    P v = st.back();
    st.pop_back();
    return v;
  };
  auto pop_mark = [&]() {
    if (marks.empty()) fail("pickle: no mark");
    const size_t m = marks.back();
    marks.pop_back();
    std::vector<P> v(st.begin() + m, st.end());
    st.resize(m);
    return v;
  };
  auto line = [&]() {
    const size_t e = d.find('\n', pc);
    if (e == std::string::npos) fail("pickle: unterminated line");
    std::string s = d.substr(pc, e - pc);
    pc = e + 1;
    return s;
  };
  auto setitems = [&](P dict, const std::vector<P>& kv) {
    if (dict->k != PV::Dict) fail("pickle: SETITEMS on a non-dict");
    for (size_t i = 0; i + 1 < kv.size(); i += 2) dict->dict.push_back({kv[i], kv[i + 1]});
  };
  while (pc < d.size()) {
    const unsigned char op = (unsigned char)d[pc++];
    switch (op) {
      case 0x80: rd(1); break;                         // PROTO
      case 0x95: rd(8); break;                         // FRAME
      case '.': return pop();                          // STOP
      case '(': marks.push_back(st.size()); break;     // MARK
      case 'N': st.push_back(mk(PV::None)); break;
      case 0x88: case 0x89: {                          // NEWTRUE / NEWFALSE
        P v = mk(PV::Bool);
        v->b = op == 0x88;
        st.push_back(v);
        break;
      }
      case 'K': case 'M': case 'J': {                  // BININT1 / BININT2 / BININT
        P v = mk(PV::Int);
        const int n = op == 'K' ? 1 : (op == 'M' ? 2 : 4);
        uint64_t u = rd(n);
        v->i = n == 4 ? (long long)(int32_t)(uint32_t)u : (long long)u;
        st.push_back(v);
        break;
      }
      case 0x8a: {                                     // LONG1
        const int n = (int)rd(1);
        long long x = 0;
        for (int q = 0; q < n; ++q) x |= (long long)(unsigned char)d[pc + q] << (8 * q);
        if (n > 0 && n < 8 && ((unsigned char)d[pc + n - 1] & 0x80)) x -= 1LL << (8 * n);
        pc += n;
        P v = mk(PV::Int);
        v->i = x;
        st.push_back(v);
        break;
      }
      case 'G': {                                      // BINFLOAT (big-endian)
        uint64_t u = 0;
        for (int q = 0; q < 8; ++q) u = (u << 8) | (unsigned char)d[pc + q];
        pc += 8;
        P v = mk(PV::Float);
        std::memcpy(&v->f, &u, 8);
        st.push_back(v);
        break;
      }
      case 'X': case 0x8c: case 'T': case 'U': case 'B': case 'C': {  // strings and bytes
        const size_t n = (op == 0x8c || op == 'U' || op == 'C') ? rd(1) : rd(4);
        if (pc + n > d.size()) fail("pickle: truncated string");
        P v = mk(PV::Str);
        v->s = d.substr(pc, n);
        pc += n;
        st.push_back(v);
        break;
      }
      case ')': st.push_back(mk(PV::Tuple)); break;    // EMPTY_TUPLE
      case ']': st.push_back(mk(PV::List)); break;     // EMPTY_LIST
      case '}': st.push_back(mk(PV::Dict)); break;     // EMPTY_DICT
      case 't': {                                      // TUPLE
        P v = mk(PV::Tuple);
        v->items = pop_mark();
        st.push_back(v);
        break;
      }
      case 0x85: case 0x86: case 0x87: {               // TUPLE1..3
        const int n = op - 0x84;
        P v = mk(PV::Tuple);
        v->items.resize(n);
        for (int q = n - 1; q >= 0; --q) v->items[q] = pop();
        st.push_back(v);
        break;
      }
      case 'l': {                                      // LIST
        P v = mk(PV::List);
        v->items = pop_mark();
        st.push_back(v);
        break;
      }
      case 'a': {                                      // APPEND
        P x = pop();
        st.back()->items.push_back(x);
        break;
      }
      case 'e': {                                      // APPENDS
        auto v = pop_mark();
        P l = st.back();
        for (auto& x : v) l->items.push_back(x);
        break;
      }
      case 's': {                                      // SETITEM
        P val = pop(), k = pop();
        setitems(st.back(), {k, val});
        break;
      }
      case 'u': {                                      // SETITEMS
        auto kv = pop_mark();
        setitems(st.back(), kv);
        break;
      }
      case 'q': memo[(long long)rd(1)] = st.back(); break;  // BINPUT
      case 'r': memo[(long long)rd(4)] = st.back(); break;  // LONG_BINPUT
      case 0x94: memo[(long long)memo.size()] = st.back(); break;  // MEMOIZE
      case 'h': case 'j': {                            // BINGET / LONG_BINGET
        const long long k = (long long)rd(op == 'h' ? 1 : 4);
        auto it = memo.find(k);
        if (it == memo.end()) fail("pickle: bad memo key");
        st.push_back(it->second);
        break;
      }
      case 'c': {                                      // GLOBAL
        P v = mk(PV::Global);
        const std::string mod = line();
        v->s = mod + " " + line();
        st.push_back(v);
        break;
      }
      case 0x81: {                                     // NEWOBJ
        P args = pop(), cls = pop();
        P o = mk(PV::Object);
        o->cls = cls;
        st.push_back(o);
        break;
      }
      case 'b': {                                      // BUILD
        P state = pop();
        P o = st.back();
        if (o->k == PV::Object) o->state = state;
        break;
      }
      case 'Q': {                                      // BINPERSID
        P pid = pop();
        if (pid->k != PV::Tuple || pid->items.size() < 5 || pid->items[0]->s != "storage")
          fail("pickle: unsupported persistent id");
        P v = mk(PV::Storage);
        v->s = pid->items[1]->s;
        v->key = pid->items[2]->s;
        v->numel = as_int(pid->items[4]);
        st.push_back(v);
        break;
      }
      case 'R': {                                      // REDUCE
        P args = pop(), fn = pop();
        const std::string g = fn->k == PV::Global ? fn->s : "";
        if (g == "torch._utils _rebuild_tensor_v2") {
          if (args->items.size() < 4) fail("pickle: bad tensor");
          P t = mk(PV::Tensor);
          t->storage = args->items[0];
          t->offset = as_int(args->items[1]);
          t->size = int_tuple(args->items[2]);
          t->stride = int_tuple(args->items[3]);
          st.push_back(t);
        } else if (g == "torch.jit._pickle restore_type_tag" || g == "torch.jit._pickle build_intlist" ||
                   g == "torch.jit._pickle build_doublelist" || g == "torch.jit._pickle build_boollist" ||
                   g == "torch.jit._pickle build_tensorlist") {
          st.push_back(args->items.empty() ? mk(PV::None) : args->items[0]);
        } else if (g == "collections OrderedDict") {
          st.push_back(mk(PV::Dict));
        } else {
          P o = mk(PV::Object);
          o->cls = fn;
          o->state = args;
          st.push_back(o);
        }
        break;
      }
      default: {
        std::ostringstream m;
        m << "pickle: unsupported opcode 0x" << std::hex << (int)op << " at " << std::dec << pc - 1;
        fail(m.str());
      }
    }
  }
  fail("pickle: no STOP");
}

// ---------------------------------------------------------------- json ---
struct JV;
using J = std::shared_ptr<JV>;
struct JV {
  enum Kind { Null, Bool, Num, Str, Arr, Obj } k = Null;
  bool b = false;
  double n = 0.0;
  std::string s;
  std::vector<J> a;
  std::map<std::string, J> o;
};

struct JsonParser {
  const std::string& t;
  size_t p = 0;
  explicit JsonParser(const std::string& s) : t(s) {}
  void ws() {
    while (p < t.size() && (t[p] == ' ' || t[p] == '\n' || t[p] == '\r' || t[p] == '\t')) ++p;
  }
  J value() {
    ws();
    if (p >= t.size()) fail("json: unexpected end");
    auto v = std::make_shared<JV>();
    const char c = t[p];
    if (c == '{') {
      v->k = JV::Obj;
      ++p;
      ws();
      if (t[p] == '}') {
        ++p;
        return v;
      }
      for (;;) {
        J key = value();
        if (key->k != JV::Str) fail("json: object key must be a string");
        ws();
        if (t[p++] != ':') fail("json: ':' expected");
        v->o[key->s] = value();
        ws();
        if (t[p] == ',') {
          ++p;
          continue;
        }
        if (t[p++] != '}') fail("json: '}' expected");
        return v;
      }
    }
    if (c == '[') {
      v->k = JV::Arr;
      ++p;
      ws();
      if (t[p] == ']') {
        ++p;
        return v;
      }
      for (;;) {
        v->a.push_back(value());
        ws();
        if (t[p] == ',') {
          ++p;
          continue;
        }
        if (t[p++] != ']') fail("json: ']' expected");
        return v;
      }
    }
    if (c == '"') {
      v->k = JV::Str;
      ++p;
      while (p < t.size() && t[p] != '"') {
        if (t[p] == '\\') {
          ++p;
          const char e = t[p];
          v->s += e == 'n' ? '\n' : e == 't' ? '\t' : e == 'r' ? '\r' : e == 'b' ? '\b' : e == 'f' ? '\f' : e;
          if (e == 'u') {  // \uXXXX: ASCII only
            v->s.back() = (char)std::stoi(t.substr(p + 1, 4), nullptr, 16);
            p += 4;
          }
          ++p;
        } else {
          v->s += t[p++];
        }
      }
      ++p;
      return v;
    }
    if (t.compare(p, 4, "true") == 0) {
      v->k = JV::Bool;
      v->b = true;
      p += 4;
      return v;
    }
    if (t.compare(p, 5, "false") == 0) {
      v->k = JV::Bool;
      p += 5;
      return v;
    }
    if (t.compare(p, 4, "null") == 0) {
      p += 4;
      return v;
    }
    size_t e = p;
    while (e < t.size() && std::strchr("+-0123456789.eE", t[e])) ++e;
    if (e == p) fail("json: unexpected character");
    v->k = JV::Num;
    v->n = std::stod(t.substr(p, e - p));
    p = e;
    return v;
  }
};

J jget(const J& o, const std::string& k) {
  if (!o || o->k != JV::Obj) return nullptr;
  auto it = o->o.find(k);
  return it == o->o.end() ? nullptr : it->second;
}
double jnum(const J& v, double dflt) { return v && v->k == JV::Num ? v->n : dflt; }
std::vector<int> jints(const J& v, std::vector<int> dflt) {
  if (!v || v->k != JV::Arr) return dflt;
  std::vector<int> out;
  for (auto& x : v->a) out.push_back((int)jnum(x, 0));
  return out;
}

}  // namespace

// ------------------------------------------------------------- model ---
struct dpgb_model_file {
  std::string def_script;
  std::vector<std::string> type_map;
  std::map<std::string, std::pair<std::vector<long long>, std::vector<double>>> tensors;  // name -> (shape, values)
  std::map<std::string, bool> flags;  // boolean attributes of the modules
  dpgb_se_a_desc desc{};
  std::vector<int> pair_mask;
  std::vector<double> bias;
  std::string type_map_text;
};

namespace {

// the object tree of data.pkl flattened to dotted names
void flatten(const P& obj, const std::string& prefix, dpgb_model_file& m,
             const std::map<std::string, ZipEntry>& zip, const std::string& buf, const std::string& root,
             int depth) {
  if (depth > 64) fail("model file: module tree too deep");
  if (!obj || obj->k != PV::Object || !obj->state || obj->state->k != PV::Dict) return;
  for (auto& kv : obj->state->dict) {
    if (!kv.first || kv.first->k != PV::Str) continue;
    const std::string name = prefix.empty() ? kv.first->s : prefix + "." + kv.first->s;
    const P& v = kv.second;
    if (!v) continue;
    if (v->k == PV::Object) {
      flatten(v, name, m, zip, buf, root, depth + 1);
    } else if (v->k == PV::Str && name == "model_def_script") {
      m.def_script = v->s;
    } else if (v->k == PV::Bool) {
      m.flags[name] = v->b;
    } else if (v->k == PV::Tensor) {
      const P& s = v->storage;
      if (!s || s->k != PV::Storage) fail("model file: tensor without storage: " + name);
      int esz = 0;
      if (s->s == "torch DoubleStorage" || s->s == "torch LongStorage") esz = 8;
      else if (s->s == "torch FloatStorage" || s->s == "torch IntStorage") esz = 4;
      else continue;  // bool / other buffers are not needed
      auto it = zip.find(root + "/data/" + s->key);
      if (it == zip.end()) fail("model file: missing storage " + s->key);
      if (it->second.method != 0) fail("model file: compressed storage " + s->key);
      long long numel = 1;
      for (long long x : v->size) numel *= x;
      std::vector<double> out((size_t)std::max(numel, 0LL));
      const int nd = (int)v->size.size();
      std::vector<long long> idx(nd, 0);
      for (long long q = 0; q < numel; ++q) {
        long long off = v->offset;
        for (int a = 0; a < nd; ++a) off += idx[a] * v->stride[a];
        if (off < 0 || (size_t)(off + 1) * esz > it->second.size) fail("model file: tensor out of its storage: " + name);
        const size_t at = it->second.data + (size_t)off * esz;
        double x;
        if (s->s == "torch DoubleStorage") {
          std::memcpy(&x, buf.data() + at, 8);
        } else if (s->s == "torch FloatStorage") {
          float y;
          std::memcpy(&y, buf.data() + at, 4);
          x = y;
        } else if (s->s == "torch LongStorage") {
          long long y;
          std::memcpy(&y, buf.data() + at, 8);
          x = (double)y;
        } else {
          int32_t y;
          std::memcpy(&y, buf.data() + at, 4);
          x = y;
        }
        out[(size_t)q] = x;
        for (int a = nd - 1; a >= 0; --a) {
          if (++idx[a] < v->size[a]) break;
          idx[a] = 0;
        }
      }
      m.tensors[name] = {v->size, std::move(out)};
    }
  }
}

const std::vector<double>* tensor(const dpgb_model_file& m, const std::string& name, bool required = true) {
  auto it = m.tensors.find(name);
  if (it == m.tensors.end()) {
    if (required) fail("model file: missing tensor " + name);
    return nullptr;
  }
  return &it->second.second;
}

// the se_e2_a description from the configuration and the weights
// (defaults of deepmd/utils/argcheck.py descrpt_se_a_args / fitting_ener)
void assemble(dpgb_model_file& m) {
  J cfg = JsonParser(m.def_script).value();
  J tm = jget(cfg, "type_map");
  if (tm && tm->k == JV::Arr)
    for (auto& x : tm->a) m.type_map.push_back(x->s);
  J de = jget(cfg, "descriptor"), fi = jget(cfg, "fitting_net");
  if (!de) fail("model file: no descriptor in model_def_script");
  J dty = jget(de, "type");
  const std::string dtype = dty ? dty->s : "";
  if (dtype != "se_e2_a" && dtype != "se_a") fail("model file: descriptor '" + dtype + "' is not se_e2_a");
  if (fi) {
    J fty = jget(fi, "type");
    if (fty && fty->s != "ener") fail("model file: fitting '" + fty->s + "' is not an energy fitting");
    if (jnum(jget(fi, "numb_fparam"), 0) != 0 || jnum(jget(fi, "numb_aparam"), 0) != 0)
      fail("model file: frame / atomic parameters are not supported");
  }
  dpgb_se_a_desc& d = m.desc;
  std::memset(&d, 0, sizeof(d));
  const std::vector<int> sel = jints(jget(de, "sel"), {});
  if (sel.empty() || (int)sel.size() > DPGB_MAX_TYPES) fail("model file: bad sel");
  d.ntypes = (int)sel.size();
  if (!m.type_map.empty() && (int)m.type_map.size() != d.ntypes) fail("model file: type_map and sel disagree");
  for (int t = 0; t < d.ntypes; ++t) d.sel[t] = sel[t];
  if (!jget(de, "rcut") || !jget(de, "rcut_smth")) fail("model file: rcut / rcut_smth missing");
  d.rcut = jnum(jget(de, "rcut"), 6.0);
  d.rcut_smth = jnum(jget(de, "rcut_smth"), 0.5);
  // the architecture from the weights themselves: the number of embedding
  // nets (ntypes: one per neighbour type; ntypes^2: per type pair), the
  // layer widths, the descriptor width of the fitting's first layer, and
  // resnet timesteps where idt tensors exist
  const std::string D = "atomic_model.descriptor.sea.", F = "atomic_model.fitting_net.";
  auto shape = [&](const std::string& n) -> const std::vector<long long>& {
    auto it = m.tensors.find(n);
    if (it == m.tensors.end()) fail("model file: missing tensor " + n);
    return it->second.first;
  };
  auto has = [&](const std::string& n) { return m.tensors.count(n) != 0; };
  auto emb = [&](int e, int l) {
    return D + "filter_layers.networks." + std::to_string(e) + ".layers." + std::to_string(l) + ".";
  };
  auto fit = [&](int t, int l) {
    return F + "filter_layers.networks." + std::to_string(t) + ".layers." + std::to_string(l) + ".";
  };
  int nnets = 0;
  while (has(emb(nnets, 0) + "matrix")) ++nnets;
  if (nnets == d.ntypes * d.ntypes && d.ntypes > 1)
    d.type_one_side = 0;
  else if (nnets == d.ntypes)
    d.type_one_side = 1;
  else
    fail("model file: " + std::to_string(nnets) + " embedding nets for " + std::to_string(d.ntypes) + " types");
  while (d.n_emb < DPGB_MAX_LAYERS && has(emb(0, d.n_emb) + "matrix")) {
    d.emb_neuron[d.n_emb] = (int)shape(emb(0, d.n_emb) + "matrix").back();
    ++d.n_emb;
  }
  if (d.n_emb == 0) fail("model file: no embedding layers");
  int nfit_layers = 0;
  while (nfit_layers <= DPGB_MAX_LAYERS && has(fit(0, nfit_layers) + "matrix")) ++nfit_layers;
  if (nfit_layers < 1) fail("model file: no fitting layers");
  d.n_fit = nfit_layers - 1;  // hidden layers; the last one is the output layer
  for (int l = 0; l < d.n_fit; ++l) d.fit_neuron[l] = (int)shape(fit(0, l) + "matrix").back();
  d.dim_descrpt = (int)shape(fit(0, 0) + "matrix").front();
  const int ng = d.emb_neuron[d.n_emb - 1];
  if (ng <= 0 || d.dim_descrpt % ng) fail("model file: descriptor width is not a multiple of the embedding width");
  d.axis_neuron = d.dim_descrpt / ng;
  d.davg = tensor(m, D + "mean")->data();
  d.dstd = tensor(m, D + "stddev")->data();
  for (int e = 0; e < nnets; ++e)
    for (int l = 0; l < d.n_emb; ++l) {
      d.emb_w[e][l] = tensor(m, emb(e, l) + "matrix")->data();
      d.emb_b[e][l] = tensor(m, emb(e, l) + "bias")->data();
      auto idt = tensor(m, emb(e, l) + "idt", false);
      d.emb_idt[e][l] = idt ? idt->data() : nullptr;
    }
  for (int t = 0; t < d.ntypes; ++t)
    for (int l = 0; l <= d.n_fit; ++l) {
      d.fit_w[t][l] = tensor(m, fit(t, l) + "matrix")->data();
      auto b = tensor(m, fit(t, l) + "bias", false);
      d.fit_b[t][l] = b ? b->data() : nullptr;
      auto idt = tensor(m, fit(t, l) + "idt", false);
      d.fit_idt[t][l] = idt ? idt->data() : nullptr;
    }
  // per-type energy bias: the fitting's bias_atom_e plus the atomic model's
  // out_bias of the energy output ([1, ntypes, 1])
  m.bias.assign(d.ntypes, 0.0);
  if (auto b = tensor(m, F + "bias_atom_e", false))
    for (int t = 0; t < d.ntypes && t < (int)b->size(); ++t) m.bias[t] += (*b)[t];
  if (auto b = tensor(m, "atomic_model.out_bias", false))
    for (int t = 0; t < d.ntypes && t < (int)b->size(); ++t) m.bias[t] += (*b)[t];
  d.atom_ener_bias = m.bias.data();
  // excluded type pairs
  J ex = jget(de, "exclude_types");
  if (ex && ex->k == JV::Arr && !ex->a.empty()) {
    m.pair_mask.assign((size_t)d.ntypes * d.ntypes, 1);
    for (auto& pr : ex->a) {
      const std::vector<int> ab = jints(pr, {});
      if (ab.size() != 2 || ab[0] < 0 || ab[1] < 0 || ab[0] >= d.ntypes || ab[1] >= d.ntypes)
        fail("model file: bad exclude_types entry");
      m.pair_mask[ab[0] * d.ntypes + ab[1]] = m.pair_mask[ab[1] * d.ntypes + ab[0]] = 0;
    }
    d.pair_mask = m.pair_mask.data();
  }
  // compressed nets (DescrptBlockSeA.enable_compression): compress_data.{e}
  // tables and compress_info.{e} = lower, upper, upper * extrapolate,
  // stride0, stride1, check_frequency
  auto cflag = m.flags.find(D + "compress");
  const bool compressed = cflag != m.flags.end() ? cflag->second
                                                 : (tensor(m, D + "compress_info.0", false) &&
                                                    tensor(m, D + "compress_info.0", false)->size() >= 6);
  if (compressed) {
    d.compressed = 1;
    for (int e = 0; e < nnets; ++e) {
      const auto* info = tensor(m, D + "compress_info." + std::to_string(e));
      if (info->size() < 6) fail("model file: bad compress_info");
      d.table[e] = tensor(m, D + "compress_data." + std::to_string(e))->data();
      for (int k = 0; k < 6; ++k) d.table_info[e][k] = (*info)[k];
    }
  }
  for (size_t t = 0; t < m.type_map.size(); ++t) m.type_map_text += (t ? " " : "") + m.type_map[t];
}

}  // namespace

extern "C" {

dpgb_model_file* dpgb_model_file_open(const char* path, const char* content, size_t size) {
  dpgb::clear_error();
  auto m = std::make_unique<dpgb_model_file>();
  try {
    std::string buf;
    if (content && size > 0) {
      buf.assign(content, size);
    } else {
      if (!path) fail("model file: no path and no content");
      std::ifstream f(path, std::ios::binary);
      if (!f) fail(std::string("model file: cannot open ") + path);
      std::ostringstream ss;
      ss << f.rdbuf();
      buf = ss.str();
    }
    const auto zip = zip_index(buf);
    std::string root, pkl;
    for (auto& kv : zip) {
      const std::string& n = kv.first;
      if (n.size() >= 9 && n.compare(n.size() - 9, 9, "/data.pkl") == 0) {
        root = n.substr(0, n.size() - 9);
        if (kv.second.method != 0) fail("model file: compressed data.pkl");
        pkl = buf.substr(kv.second.data, kv.second.size);
        break;
      }
    }
    if (pkl.empty()) fail("model file: no data.pkl (not a TorchScript archive)");
    P top = unpickle(pkl);
    flatten(top, "", *m, zip, buf, root, 0);
    if (m->def_script.empty()) fail("model file: no model_def_script");
    assemble(*m);
  } catch (const Fail& f) {
    set_error(f.msg);
    return nullptr;
  } catch (const std::exception& e) {
    set_error(std::string("model file: ") + e.what());
    return nullptr;
  }
  return m.release();
}

void dpgb_model_file_close(dpgb_model_file* m) { delete m; }

const dpgb_se_a_desc* dpgb_model_file_desc(const dpgb_model_file* m) { return m ? &m->desc : nullptr; }

const char* dpgb_model_file_type_map(const dpgb_model_file* m) { return m ? m->type_map_text.c_str() : ""; }

const char* dpgb_model_file_config(const dpgb_model_file* m) { return m ? m->def_script.c_str() : ""; }

long long dpgb_model_file_tensor(const dpgb_model_file* m, const char* name, double* out, long long cap,
                                 long long* shape, int* ndim) {
  dpgb::clear_error();
  if (!m || !name) {
    set_error("NULL model file or name");
    return -1;
  }
  auto it = m->tensors.find(name);
  if (it == m->tensors.end()) {
    set_error(std::string("no tensor ") + name);
    return -1;
  }
  const auto& sh = it->second.first;
  const auto& v = it->second.second;
  if (ndim) {
    const int cap_dims = *ndim;
    *ndim = (int)sh.size();
    if (shape)
      for (int a = 0; a < (int)sh.size() && a < cap_dims; ++a) shape[a] = sh[a];
  }
  if (out)
    for (long long q = 0; q < (long long)v.size() && q < cap; ++q) out[q] = v[(size_t)q];
  return (long long)v.size();
}

}  // extern "C"

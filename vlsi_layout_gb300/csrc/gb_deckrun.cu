// gb_deckrun.cu -- the MAGPARSER control-deck interpreter on the GPU engine.
//
// Follows ParseControlFile (controlparser.f90:116-654): one statement per line,
// keywords program / var / decl / exec / systeminfo / info / flush / delete /
// end, '#' comments.  Designs are declared from Magic files
// (`decl design d1 = X.mag`, parsed like parseMagicLayoutFile,
// magparser.f90:108-482: `<< layer >>` sections with `rect x1 y1 x2 y2` lines,
// `KLBIN path` and `SNAP path` lines), as outputs written on flush
// (`decl output o1 = Y.mag`), or as memory designs (`decl memory t1 =
// nothing`).  Layer files follow RestoreSnapToLayer (diskdesign_impl.f90:
// 83-113): a path containing ".bin" is a KLBin file (raw int32x4, an invalid
// box refuses the file, kldata.f90:14-60), any other path a .snap file; with
// `var temporary_layers 2` a missing file is an empty layer.  On flush
// (magparser.f90:510-560, controlparser.f90:613-625) output layers go to the
// files their Y.mag names (".snap": SaveLayerToSnap with method 1, ".bin":
// KLBin), and with temporary_layers 2 memory layers go to SNAP files named
// temp_folder + design + "_MTL_" + layer (controlparser.f90:335,374); a
// flushed layer leaves the device and is restored from its file when a later
// statement reads it.  `exec run LHS = RHS1 OP RHS2 [args]` dispatches the
// operators of controlparser.f90:442-585 to device-resident layers:
//   + OR, * AND, @ ~ ! NOT / FRAMENOT, ^ XOR (abort_on_xor), % no-op,
//   OR2 AND2 NOT FRAMENOT XOR, AND (single layer: covered twice), GROW e n w s,
//   SIZE r, EXTENT, COPY,
//   ASSERT_ZERO, WORMHOLE (no-op).
// GROW / SIZE amounts are um, converted with int(1000*r) (truncation).  The
// README's RUN_LOOP(`OP1', ...) macro line (op_template.m4) is expanded in
// place, so the README deck runs without m4.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "gbool.h"
#include "gb_internal.h"

namespace {

struct DeckLayer {
  gb_layer* L = nullptr;
  std::string backing;   // the layer's file: KLBIN / SNAP path of its .mag, or a memory layer's SNAP file
  bool flushed = false;  // written to `backing` and dropped from the device; restored when next read
};

struct Design {
  std::string name, file;
  int dir = 0;              // 0 input, 1 output, 2 memory
  bool mag_parsed = false;  // output: its .mag existed and named the layers' files
  std::vector<std::string> order;
  std::map<std::string, DeckLayer> layers;
};

struct Deck {
  gb_context* ctx = nullptr;
  std::map<std::string, Design> dbs;
  std::string log;
  std::string base_dir;
  std::string temp_folder;  // var temp_folder: prefix of memory layers' files (controlparser.f90:182-187)
  int abort_on_xor = 0, abort_on_assert_zero = 0, verbosity = 0, temporary_layers = 0;
  int assert_failures = 0;
  int line_no = 0;
  std::vector<c_box> empty;
  std::vector<gb_layer*> owned;  // raw layers created by the interpreter

  void say(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    log += buf;
    log += "\n";
  }
};

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

std::vector<std::string> split_ws(const std::string& s) {
  std::istringstream is(s);
  std::vector<std::string> v;
  std::string t;
  while (is >> t) v.push_back(t);
  return v;
}

bool file_exists(const std::string& f) {
  FILE* fp = fopen(f.c_str(), "rb");
  if (!fp) return false;
  fclose(fp);
  return true;
}

bool ends_with(const std::string& s, const std::string& t) {
  return s.size() >= t.size() && s.compare(s.size() - t.size(), t.size(), t) == 0;
}

// A relative path names a file in the working directory when it exists there,
// else in the deck's directory.
std::string resolve(const Deck& d, const std::string& f) {
  if (f.empty() || f[0] == '/') return f;
  if (file_exists(f)) return f;
  return d.base_dir + "/" + f;
}

int make_layer(Deck& d, const c_box* boxes, size_t n, gb_layer** out) {
  int e = gb_layer_from_host(d.ctx, n ? boxes : nullptr, n, nullptr, 1, out);
  if (!e) d.owned.push_back(*out);
  return e;
}
int make_layer(Deck& d, const std::vector<c_box>& boxes, gb_layer** out) {
  return make_layer(d, boxes.data(), boxes.size(), out);
}

// LoadKLBin (kldata.f90:14-60): the whole file in one read into pinned host
// memory and one upload; an empty or missing file and any invalid box refuse
// the file, as the reference's error stops do.
int read_klbin(Deck& d, const std::string& path, gb_layer** out) {
  FILE* fp = fopen(path.c_str(), "rb");
  long long bytes = -1;
  if (fp && fseek(fp, 0, SEEK_END) == 0) bytes = ftell(fp);
  if (!fp || bytes <= 0) {
    if (fp) fclose(fp);
    d.say("ERROR: KLBIN File %s is empty or does not exist.", path.c_str());
    return GB_ERR_ARG;
  }
  fseek(fp, 0, SEEK_SET);
  const long long n = bytes / (long long)sizeof(c_box);
  c_box* h = nullptr;
  const bool pinned = cudaMallocHost((void**)&h, (size_t)std::max(1ll, n) * sizeof(c_box)) == cudaSuccess;
  if (!pinned) {
    cudaGetLastError();
    h = (c_box*)malloc((size_t)std::max(1ll, n) * sizeof(c_box));
  }
  int e = GB_OK;
  if (!h || (long long)fread(h, sizeof(c_box), (size_t)n, fp) != n) {
    d.say("ERROR: cannot read KLBIN %s", path.c_str());
    e = GB_ERR_ARG;
  }
  fclose(fp);
  for (long long i = 0; i < n && !e; ++i) {
    if (!(h[i].x1 < h[i].x2 && h[i].y1 < h[i].y2)) {  // Box%is_valid, geometry.f90:66-70
      d.say("ERROR: INVALID BOX detected on input: box %lld (%d %d %d %d) of %s", i + 1, h[i].x1, h[i].y1, h[i].x2,
            h[i].y2, path.c_str());
      e = GB_ERR_INVALID_BOX;
    }
  }
  if (!e) e = make_layer(d, h, (size_t)n, out);
  if (pinned) cudaFreeHost(h);
  else free(h);
  return e;
}

// A .snap file decoded on the device (gb_restore_snap_to_layer) into a layer.
int read_snap_layer(Deck& d, const std::string& path, gb_layer** out) {
  long long n = 0, nch = 0;
  int method = 0, props = 0;
  int e = gb_snap_file_info(path.c_str(), &n, &nch, &method, &props);
  if (e) {
    d.say("ERROR: cannot read SNAP file %s (status %d)", path.c_str(), e);
    return e;
  }
  if (n == 0) return make_layer(d, d.empty, out);
  c_box* db = nullptr;
  if (cudaMalloc((void**)&db, (size_t)n * sizeof(c_box)) != cudaSuccess) {
    cudaGetLastError();
    return GB_ERR_OOM;
  }
  long long got = 0;
  e = gb_restore_snap_to_layer(d.ctx, path.c_str(), db, n, &got, nullptr);
  if (!e && got != n) e = GB_ERR_CORRUPT;  // diskdesign_impl.f90:104-109: SNAP RESTORATION FAILED
  if (!e) {
    e = gb_layer_from_device(d.ctx, db, (unsigned long long)n, nullptr, 1, out);
    if (!e) {
      d.owned.push_back(*out);
      e = gb_sync(d.ctx, nullptr);
    }
  }
  if (e) d.say("ERROR: SNAP restoration failed for file: %s (%s)", path.c_str(), gb_last_error(d.ctx));
  cudaFree(db);
  return e;
}

// RestoreSnapToLayer (diskdesign_impl.f90:83-113).
int restore_layer(Deck& d, const std::string& name, gb_layer** out) {
  const std::string path = resolve(d, name);
  if (d.temporary_layers > 1 && !file_exists(path)) return make_layer(d, d.empty, out);  // no file: empty layer
  if (name.find(".bin") != std::string::npos) return read_klbin(d, path, out);
  return read_snap_layer(d, path, out);
}

// Boxes of a device layer on the host.
int layer_boxes(Deck& d, gb_layer* L, std::vector<c_box>& v) {
  unsigned long long n = 0;
  int e = gb_layer_to_host(d.ctx, L, nullptr, 0, &n, nullptr);
  if (e && e != GB_ERR_CAPACITY) return e;
  v.resize(n);
  return gb_layer_to_host(d.ctx, L, v.data(), n, &n, nullptr);
}

// parseMagicLayoutFile (magparser.f90:108-482).  Input designs load their
// layers; an output design only records where each layer is to be written.
int load_mag(Deck& d, Design& D) {
  std::ifstream in(resolve(d, D.file));
  if (!in.good()) {
    if (D.dir == 1) return GB_OK;  // no output .mag yet: flush writes a new one
    d.say("ERROR: cannot open %s", D.file.c_str());
    return GB_ERR_ARG;
  }
  if (D.dir == 1) D.mag_parsed = true;
  std::map<std::string, std::vector<c_box>> boxes;  // rect lines (after the layer's file line, if any)
  std::map<std::string, std::string> src;           // KLBIN / SNAP file of the layer
  std::string line, section;
  while (std::getline(in, line)) {
    line = trim(line);
    if (line.rfind("<< end >>", 0) == 0) break;
    if (line.rfind("<<", 0) == 0) {
      size_t e = line.find(">>");
      section = trim(line.substr(2, e == std::string::npos ? std::string::npos : e - 2));
      if (section != "labels" && section != "properties" && !boxes.count(section)) {
        boxes[section];
        D.order.push_back(section);
      }
      continue;
    }
    if (section.empty() || section == "labels" || section == "properties") continue;
    if (line.rfind("rect", 0) == 0) {
      std::vector<std::string> t = split_ws(line);
      if (t.size() >= 5) {
        c_box b{(int32_t)atol(t[1].c_str()), (int32_t)atol(t[2].c_str()), (int32_t)atol(t[3].c_str()),
                (int32_t)atol(t[4].c_str())};
        if (!(b.x1 < b.x2 && b.y1 < b.y2)) {  // addBoxToLayer's CheckBox, magparser.f90:497-499
          d.say("ERROR: box in valid: %s (%s)", line.c_str(), D.file.c_str());
          return GB_ERR_INVALID_BOX;
        }
        boxes[section].push_back(b);
      }
    } else if (line.rfind("KLBIN", 0) == 0 || line.rfind("SNAP", 0) == 0) {
      std::vector<std::string> t = split_ws(line);
      if (t.size() >= 2) {
        src[section] = t[1];
        boxes[section].clear();  // the file replaces the layer's boxes (magparser.f90:243-246)
      }
    }
  }
  for (const std::string& name : D.order) {
    DeckLayer& DL = D.layers[name];
    if (src.count(name)) DL.backing = src[name];
    if (D.dir == 1) continue;
    gb_layer* L = nullptr;
    int e = GB_OK;
    if (src.count(name)) {
      e = restore_layer(d, src[name], &L);
      if (!e && !boxes[name].empty()) {  // rect lines after the file line add to it
        std::vector<c_box> v;
        e = layer_boxes(d, L, v);
        v.insert(v.end(), boxes[name].begin(), boxes[name].end());
        if (!e) e = make_layer(d, v, &L);
      }
    } else {
      e = make_layer(d, boxes[name], &L);
    }
    if (e) return e;
    DL.L = L;
    long long n = 0;
    gb_layer_count(d.ctx, L, &n, nullptr);
    d.say("  layer %-12s %8lld boxes%s%s", name.c_str(), n, src.count(name) ? " from " : "",
          src.count(name) ? src[name].c_str() : "");
  }
  return GB_OK;
}

// SaveLayerToSnap (diskdesign_impl.f90:59-81) with method 1, or WriteKLBin
// (kldata.f90:61-98) in one write.
int save_layer(Deck& d, gb_layer* L, const std::string& path, bool snap) {
  if (snap) {
    const c_box* db = nullptr;
    long long n = 0;
    int e = gbi::layer_device_boxes(d.ctx, L, &db, &n);
    if (!e) e = gb_save_layer_to_snap(d.ctx, path.c_str(), db, n, 1, 0, nullptr);
    if (e) d.say("ERROR: cannot write SNAP file %s (%s)", path.c_str(), gb_last_error(d.ctx));
    return e;
  }
  std::vector<c_box> v;
  int e = layer_boxes(d, L, v);
  if (e) return e;
  FILE* fp = fopen(path.c_str(), "wb");
  if (!fp || fwrite(v.data(), sizeof(c_box), v.size(), fp) != v.size()) {
    if (fp) fclose(fp);
    d.say("ERROR: cannot write KLBIN file %s", path.c_str());
    return GB_ERR_ARG;
  }
  fclose(fp);
  return GB_OK;
}

// ClearLayer after a flush: the device copy goes, the file stays.
void drop_layer(Deck& d, DeckLayer& DL) {
  auto it = std::find(d.owned.begin(), d.owned.end(), DL.L);
  if (it != d.owned.end()) {
    gb_layer_free(d.ctx, DL.L);
    d.owned.erase(it);
  }
  DL.L = nullptr;
  DL.flushed = true;
}

// An output design whose .mag did not exist: a new .mag with rect lines, and
// SNAP side files for large layers.
int write_new_mag(Deck& d, Design& D) {
  const std::string path = D.file;
  FILE* fp = fopen(path.c_str(), "w");
  if (!fp) {
    d.say("ERROR: cannot write %s", path.c_str());
    return GB_ERR_ARG;
  }
  fprintf(fp, "magic\ntech gb300\n");
  for (const std::string& name : D.order) {
    gb_layer* L = D.layers[name].L;
    if (!L) continue;
    long long n = 0;
    int e = gb_layer_count(d.ctx, L, &n, nullptr);
    if (e) { fclose(fp); return e; }
    fprintf(fp, "<< %s >>\n", name.c_str());
    if (n > 100000) {
      const std::string side = path + "_" + name + ".snap";
      e = save_layer(d, L, side, true);
      if (e) { fclose(fp); return e; }
      fprintf(fp, "SNAP %s\n", side.c_str());
    } else {
      std::vector<c_box> v;
      e = layer_boxes(d, L, v);
      if (e) { fclose(fp); return e; }
      for (const c_box& b : v) fprintf(fp, "rect %d %d %d %d\n", b.x1, b.y1, b.x2, b.y2);
    }
  }
  fprintf(fp, "<< end >>\n");
  fclose(fp);
  d.say("  wrote %s", path.c_str());
  return GB_OK;
}

// writeMagicLayoutFile (magparser.f90:510-560) for one design.
int flush_design(Deck& d, Design& D) {
  if (D.dir == 1 && !D.mag_parsed) return write_new_mag(d, D);
  for (const std::string& name : D.order) {
    DeckLayer& DL = D.layers[name];
    if (!DL.L) continue;
    long long n = 0;
    int e = gb_layer_count(d.ctx, DL.L, &n, nullptr);
    if (e) return e;
    if (n == 0) continue;  // empty layers are not written
    std::string file = DL.backing;
    bool snap = true;
    if (D.dir == 2) {
      file = d.temp_folder + D.name + "_MTL_" + name;  // controlparser.f90:335,374
      DL.backing = file;
    } else if (ends_with(file, ".snap")) {
      snap = true;
    } else if (ends_with(file, ".bin")) {
      snap = false;
    } else {
      d.say("ERROR: File format not supported: %s (layer %s): DBOUT only supports KLBIN", file.c_str(), name.c_str());
      return GB_ERR_ARG;
    }
    e = save_layer(d, DL.L, file, snap);
    if (e) return e;
    d.say("  wrote %s:%s (%lld boxes) to %s", D.name.c_str(), name.c_str(), n, file.c_str());
    drop_layer(d, DL);
  }
  return GB_OK;
}

bool split_ref(const std::string& s, std::string& db, std::string& layer) {
  size_t p = s.find(':');
  if (p == std::string::npos) return false;
  db = s.substr(0, p);
  layer = s.substr(p + 1);
  return true;
}

gb_layer* lookup(Deck& d, const std::string& ref, bool& ok, int* err = nullptr) {
  std::string db, ly;
  ok = false;
  if (!split_ref(ref, db, ly) || !d.dbs.count(db)) return nullptr;
  Design& D = d.dbs[db];
  if (!D.layers.count(ly)) return nullptr;
  DeckLayer& DL = D.layers[ly];
  if (DL.flushed && !DL.L) {  // controlparser.f90:440-441: a flushed layer is read back from its file
    gb_layer* L = nullptr;
    const int e = restore_layer(d, DL.backing, &L);
    if (e) {
      if (err) *err = e;
      return nullptr;
    }
    DL.L = L;
    DL.flushed = false;
  }
  ok = true;
  return DL.L;
}

void assign(Deck& d, const std::string& ref, gb_layer* L) {
  std::string db, ly;
  split_ref(ref, db, ly);
  Design& D = d.dbs[db];
  if (!D.layers.count(ly)) D.order.push_back(ly);
  D.layers[ly].L = L;
  D.layers[ly].flushed = false;
}

int count_of(Deck& d, gb_layer* L, long long* n) { return gb_layer_count(d.ctx, L, n, nullptr); }

// One `exec run` statement.
int exec_run(Deck& d, const std::string& rest) {
  const size_t eq = rest.find('=');
  if (eq == std::string::npos) {
    d.say("Syntax ERROR: line %d", d.line_no);
    return GB_ERR_ARG;
  }
  const std::string lhs = trim(rest.substr(0, eq));
  std::vector<std::string> t = split_ws(rest.substr(eq + 1));
  if (t.size() < 3) {
    d.say("Syntax ERROR: line %d", d.line_no);
    return GB_ERR_ARG;
  }
  std::string db, ly;
  if (!split_ref(lhs, db, ly) || !d.dbs.count(db)) {
    d.say("ERROR: LHS db not found: %s (line %d)", lhs.c_str(), d.line_no);
    return GB_ERR_ARG;
  }
  bool ok1 = false, ok2 = false;
  int lerr = GB_OK;
  gb_layer* A = lookup(d, t[0], ok1, &lerr);
  if (lerr) return lerr;
  if (!ok1) {
    d.say("ERROR: layer not found: %s (line %d)", t[0].c_str(), d.line_no);  // controlparser.f90:401-405
    return GB_ERR_ARG;
  }
  const std::string op = t[1];
  gb_layer* B = nullptr;
  const bool nothing = t[2] == "nothing" || t[2].find(":nothing") != std::string::npos;
  if (!nothing) {
    B = lookup(d, t[2], ok2, &lerr);
    if (lerr) return lerr;
    if (!ok2) {
      d.say("ERROR: layer not found: %s (line %d)", t[2].c_str(), d.line_no);
      return GB_ERR_ARG;
    }
  }
  // a binary operator whose second operand is `nothing` sees an empty layer
  // (the reference's init layer `t1:nothing` holds no boxes)
  auto need_b = [&]() {
    if (!B && nothing) {
      if (make_layer(d, d.empty, &B)) B = nullptr;
    }
    if (!B) d.say("ERROR: operator %s needs a second layer (line %d)", op.c_str(), d.line_no);
    return B != nullptr;
  };
  gb_layer* O = nullptr;
  int e = GB_OK;
  if (op == "+" || op == "OR2") {
    if (!need_b()) return GB_ERR_ARG;
    e = gb_op_bool(d.ctx, GB_OP_OR, A, B, &O);
  } else if (op == "*" || op == "AND2") {
    if (!need_b()) return GB_ERR_ARG;
    e = gb_op_bool(d.ctx, GB_OP_AND, A, B, &O);
  } else if (op == "@" || op == "~" || op == "!" || op == "NOT" || op == "FRAMENOT") {
    if (!need_b()) return GB_ERR_ARG;
    e = gb_op_bool(d.ctx, GB_OP_NOT, A, B, &O);
  } else if (op == "AND") {  // single-layer AND (controlparser.f90:545-549, design_impl.f90:385-498)
    e = gb_op_bool(d.ctx, GB_OP_OVERLAP, A, nullptr, &O);
  } else if (op == "^" || op == "XOR") {
    if (!need_b()) return GB_ERR_ARG;
    e = gb_op_bool(d.ctx, GB_OP_XOR, A, B, &O);
    long long n = 0;
    if (!e) e = count_of(d, O, &n);
    if (!e && op == "^" && d.abort_on_xor > 0 && n > 0) {  // controlparser.f90:472-475
      d.say("ERROR: Aborting RUN since abort_on_xor set > 0, and ^ layer has %lld shapes.", n);
      assign(d, lhs, O);
      return GB_ERR_ARG;
    }
  } else if (op == "%" || op == "WORMHOLE") {
    return GB_OK;
  } else if (op == "ASSERT_ZERO") {
    long long n = 0;
    e = count_of(d, A, &n);
    if (e) return e;
    if (n > 0) {  // controlparser.f90:524-530
      ++d.assert_failures;
      d.say("************ ASSERT_ZERO fail on layer %s (%lld boxes). Line: %d **********************",
            t[0].c_str(), n, d.line_no);
      if (d.abort_on_assert_zero > 1) return GB_ERR_ARG;
    } else {
      d.say("  ASSERT_ZERO %s: pass", t[0].c_str());
    }
    return GB_OK;
  } else if (op == "GROW") {
    if (t.size() < 7) {
      d.say("Syntax ERROR: GROW needs 4 amounts (line %d)", d.line_no);
      return GB_ERR_ARG;
    }
    int32_t v[4];
    for (int k = 0; k < 4; ++k) v[k] = gb_um_to_dbu(strtod(t[3 + k].c_str(), nullptr));
    e = gb_op_grow(d.ctx, A, v[0], v[1], v[2], v[3], &O);
  } else if (op == "SIZE") {
    if (t.size() < 4) {
      d.say("Syntax ERROR: SIZE needs an amount (line %d)", d.line_no);
      return GB_ERR_ARG;
    }
    e = gb_op_size(d.ctx, A, gb_um_to_dbu(strtod(t[3].c_str(), nullptr)), &O);
  } else if (op == "COPY") {
    e = gb_op_bool(d.ctx, GB_OP_MERGE, A, nullptr, &O);
  } else if (op == "EXTENT") {
    unsigned long long n = 0;
    e = gb_layer_to_host(d.ctx, A, nullptr, 0, &n, nullptr);
    if (e && e != GB_ERR_CAPACITY) return e;
    std::vector<c_box> v(n);
    e = gb_layer_to_host(d.ctx, A, v.data(), n, &n, nullptr);
    if (e) return e;
    std::vector<c_box> bb;
    if (n) {
      c_box x = v[0];
      for (const c_box& b : v) {
        x.x1 = std::min(x.x1, b.x1); x.y1 = std::min(x.y1, b.y1);
        x.x2 = std::max(x.x2, b.x2); x.y2 = std::max(x.y2, b.y2);
      }
      bb.push_back(x);
    }
    e = make_layer(d, bb, &O);
  } else {
    if (op == "GRID")  // controlparser.f90:559-562 calls CreateGRID, which no source file defines
      d.say("ERROR: GRID has no definition in the control language's sources (line %d)", d.line_no);
    else
      d.say("UNKNOWN primary_operator: %s on line: %d", op.c_str(), d.line_no);
    return GB_ERR_ARG;
  }
  if (e) {
    d.say("ERROR: operator %s failed with status %d (%s), line %d", op.c_str(), e, gb_last_error(d.ctx),
          d.line_no);
    return e;
  }
  assign(d, lhs, O);
  if (d.verbosity > 0) {
    long long n = 0;
    count_of(d, O, &n);
    d.say("  %s = %s %s %s : %lld boxes", lhs.c_str(), t[0].c_str(), op.c_str(), t[2].c_str(), n);
  }
  return gb_sync(d.ctx, nullptr);
}

// RUN_LOOP(`OP1',`t',`d',`layer',`amount', ...) -> the eight OP1 statements
// per (layer, amount) pair (op_template.m4:10-22).
bool expand_run_loop(const std::string& line, std::vector<std::string>& out) {
  if (line.rfind("RUN_LOOP(", 0) != 0) return false;
  std::string body = line.substr(9);
  size_t e = body.rfind(')');
  if (e != std::string::npos) body = body.substr(0, e);
  std::vector<std::string> a;
  std::string cur;
  for (char ch : body) {
    if (ch == ',') { a.push_back(trim(cur)); cur.clear(); }
    else if (ch != '`' && ch != '\'') cur += ch;
  }
  a.push_back(trim(cur));
  if (a.size() < 5 || a[0] != "OP1") return false;
  const std::string t = a[1], dsg = a[2];
  for (size_t k = 3; k + 1 < a.size(); k += 2) {
    const std::string L = a[k], r = a[k + 1];
    if (L.empty()) break;
    out.push_back("exec run " + t + ":" + L + "_1 = " + dsg + ":" + L + " GROW " + t + ":nothing " + r + " " + r +
                  " " + r + " " + r);
    out.push_back("exec run " + t + ":" + L + "_2 = " + dsg + ":" + L + " SIZE " + t + ":nothing -" + r);
    out.push_back("exec run " + t + ":" + L + "_outer_ring = " + t + ":" + L + "_1 ~ " + dsg + ":" + L);
    out.push_back("exec run " + t + ":" + L + "_inner_ring = " + dsg + ":" + L + " ~ " + t + ":" + L + "_2");
    out.push_back("exec run " + t + ":" + L + "_ring_and1 = " + t + ":" + L + "_outer_ring * " + dsg + ":" + L);
    out.push_back("exec run " + t + ":" + L + "_ring_intersection = " + t + ":" + L + "_outer_ring * " + t + ":" + L +
                  "_inner_ring");
    out.push_back("exec run " + t + ":nothing = " + t + ":" + L + "_ring_and1 ASSERT_ZERO " + t + ":nothing");
    out.push_back("exec run " + t + ":nothing = " + t + ":" + L + "_ring_intersection ASSERT_ZERO " + t + ":nothing");
  }
  return true;
}

int run_lines(Deck& d, const std::vector<std::string>& lines) {
  for (size_t li = 0; li < lines.size(); ++li) {
    d.line_no = (int)li + 1;
    std::string line = trim(lines[li]);
    if (line.empty() || line[0] == '#' || line.rfind("dnl", 0) == 0 || line.rfind("include(", 0) == 0) continue;
    std::vector<std::string> exp;
    if (expand_run_loop(line, exp)) {
      for (const std::string& x : exp) {
        const size_t p = x.find(' ');
        const std::string r = trim(x.substr(p + 1));
        int e = exec_run(d, trim(r.substr(r.find(' ') + 1)));
        if (e) return e;
      }
      continue;
    }
    const size_t p = line.find(' ');
    const std::string kw = p == std::string::npos ? line : line.substr(0, p);
    const std::string rest = p == std::string::npos ? "" : trim(line.substr(p + 1));
    if (kw == "program") {
      d.say("--- Starting Program: %s", rest.c_str());
    } else if (kw == "var") {
      std::vector<std::string> t = split_ws(rest);
      if (t.size() >= 2) {
        const int v = atoi(t[1].c_str());
        if (t[0] == "temp_folder") d.temp_folder = t[1];
        else if (t[0] == "abort_on_xor") d.abort_on_xor = v;
        else if (t[0] == "abort_on_assert_zero") d.abort_on_assert_zero = v;
        else if (t[0] == "debug_verbosity") d.verbosity = v;
        else if (t[0] == "temporary_layers") d.temporary_layers = v;
        // gpu is accepted; the GPU engine is the only back end here
      }
    } else if (kw == "decl") {
      std::vector<std::string> t = split_ws(rest);
      if (t.size() < 4 || t[2] != "=") {
        d.say("Syntax ERROR: line %d", d.line_no);
        return GB_ERR_ARG;
      }
      Design D;
      D.name = t[1];
      D.file = t[3];
      if (t[0] == "design") {
        D.dir = 0;
        d.say("decl design %s = %s", D.name.c_str(), D.file.c_str());
        int e = load_mag(d, D);
        if (e) return e;
      } else if (t[0] == "output") {
        D.dir = 1;
        int e = load_mag(d, D);  // records each layer's file (controlparser.f90:238-256)
        if (e) return e;
      } else if (t[0] == "memory") {
        if (t[3] != "nothing") {
          d.say("MEMORY DB must have backing store nothing (line %d)", d.line_no);
          return GB_ERR_ARG;
        }
        D.dir = 2;
      } else {
        d.say("Syntax ERROR: line %d", d.line_no);
        return GB_ERR_ARG;
      }
      d.dbs[D.name] = D;
    } else if (kw == "exec") {
      const size_t q = rest.find(' ');
      const std::string sub = rest.substr(0, q);
      const std::string arg = q == std::string::npos ? "" : trim(rest.substr(q + 1));
      if (sub == "init") {
        std::string db, ly;
        if (!split_ref(split_ws(arg)[0], db, ly) || !d.dbs.count(db)) {
          d.say("DB: %s not found. Syntax ERROR: line %d", arg.c_str(), d.line_no);
          return GB_ERR_ARG;
        }
        gb_layer* L = nullptr;
        int e = make_layer(d, d.empty, &L);
        if (e) return e;
        assign(d, split_ws(arg)[0], L);
      } else if (sub == "run") {
        int e = exec_run(d, arg);
        if (e) return e;
      } else {
        d.say("Syntax ERROR: line %d", d.line_no);
        return GB_ERR_ARG;
      }
    } else if (kw == "flush") {  // controlparser.f90:613-625
      for (auto& kv : d.dbs) {
        Design& D = kv.second;
        if (D.dir == 1 || (D.dir == 2 && d.temporary_layers == 2)) {
          int e = flush_design(d, D);
          if (e) return e;
        }
      }
    } else if (kw == "delete") {
      d.dbs.erase(split_ws(rest).empty() ? "" : split_ws(rest)[0]);
    } else if (kw == "systeminfo" || kw == "info") {
      size_t fr = 0, tot = 0;
      cudaMemGetInfo(&fr, &tot);
      d.say("--- %s: device memory free %.1f GiB of %.1f GiB", kw.c_str(), fr / 1073741824.0, tot / 1073741824.0);
    } else if (kw == "end") {
      d.say("--- End of file");
      break;
    } else {
      d.say("Unknown command: %s", kw.c_str());
    }
  }
  return GB_OK;
}

}  // namespace

extern "C" int gb_run_deck(const char* path, char* log, unsigned long long log_cap, int* assert_failures) {
  if (!path) return GB_ERR_ARG;
  std::ifstream in(path);
  if (!in.good()) return GB_ERR_ARG;
  std::vector<std::string> lines;
  std::string line;
  while (std::getline(in, line)) lines.push_back(line);
  Deck d;
  const std::string p(path);
  const size_t sl = p.rfind('/');
  d.base_dir = sl == std::string::npos ? "." : p.substr(0, sl);
  int dev = 0;
  cudaGetDevice(&dev);
  int e = gb_context_create(dev, 0, &d.ctx);
  if (e) return e;
  e = run_lines(d, lines);
  if (assert_failures) *assert_failures = d.assert_failures;
  if (log && log_cap) {
    const size_t n = std::min<size_t>(d.log.size(), log_cap - 1);
    memcpy(log, d.log.data(), n);
    log[n] = 0;
  }
  for (gb_layer* L : d.owned) gb_layer_free(d.ctx, L);
  gb_context_destroy(d.ctx);
  return e;
}

// Scene files: the reference's `.ribo` format (src/world/snapshot.rs:1-10,
// 110-136, 144-167) for the world blocks of this path.
//
// Layout: "RIBOSCN1", u32 header length, a JSON header, then blocks of
// (u16 name length, name, u64 stored length, stored bytes), each block's
// bytes being a u32 uncompressed length followed by one LZ4 block.  The
// reference reads the header's "cfg" (sizes must match), "params" (SimParams
// by field name: unknown names ignored, missing ones at their defaults) and
// "settings", and the blocks chem, gamma, velocity, pressure, temperature and
// redox, plus its agent blocks.  A scene written here has zero agents (empty
// agent blocks, so the reference loads it into any world of the same size),
// and three blocks of its own (gb300_heat, gb300_light, gb300_shade: this
// path's frozen inputs) that the reference ignores; "gb300_settings" in the
// header carries this path's settings.
//
// The LZ4 block coder follows the published LZ4 block format (sequences of a
// token, literal run, 16-bit little-endian match offset and match length;
// matches of at least 4 bytes; the last 5 bytes literals; no match starting
// within 12 bytes of the end).  The JSON reader is a small recursive-descent
// parser over the whole header (values it does not use are skipped).
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/ribo_world.h"
#include "ribo_world_impl.h"

namespace ribo {
namespace {

// ---------------------------------------------------------------------------
// LZ4 block format.
constexpr size_t LZ_MINMATCH = 4, LZ_LASTLITERALS = 5, LZ_MFLIMIT = 12;
constexpr int LZ_HASH_LOG = 16;

inline uint32_t load32(const uint8_t* p) {
  uint32_t v;
  memcpy(&v, p, 4);
  return v;
}
inline uint32_t lz_hash(uint32_t v) { return (v * 2654435761u) >> (32 - LZ_HASH_LOG); }

void put_length(std::vector<uint8_t>& out, size_t extra) {  // the 255-run after a 15 nibble
  while (extra >= 255) {
    out.push_back(255);
    extra -= 255;
  }
  out.push_back((uint8_t)extra);
}
void put_sequence(std::vector<uint8_t>& out, const uint8_t* lit, size_t nlit, size_t offset, size_t mlen) {
  const size_t tok_at = out.size();
  out.push_back(0);
  uint8_t tok = (uint8_t)((nlit >= 15 ? 15 : nlit) << 4);
  if (nlit >= 15) put_length(out, nlit - 15);
  out.insert(out.end(), lit, lit + nlit);
  if (mlen) {
    out.push_back((uint8_t)(offset & 0xff));
    out.push_back((uint8_t)(offset >> 8));
    const size_t ml = mlen - LZ_MINMATCH;
    tok |= (uint8_t)(ml >= 15 ? 15 : ml);
    if (ml >= 15) put_length(out, ml - 15);
  }
  out[tok_at] = tok;
}

// Greedy single-pass compressor: a hash table of the last position of each
// 4-byte sequence; the longest forward extension of a verified candidate.
void lz4_compress(const uint8_t* src, size_t n, std::vector<uint8_t>& out) {
  out.clear();
  out.reserve(n + n / 255 + 16);
  size_t anchor = 0;
  if (n > LZ_MFLIMIT) {
    std::vector<int64_t> table((size_t)1 << LZ_HASH_LOG, -1);
    const size_t last_start = n - LZ_MFLIMIT;    // a match starts at or before this
    const size_t match_end = n - LZ_LASTLITERALS;  // and ends at or before this
    size_t ip = 0;
    while (ip <= last_start) {
      const uint32_t seq = load32(src + ip);
      const uint32_t h = lz_hash(seq);
      const int64_t ref = table[h];
      table[h] = (int64_t)ip;
      if (ref >= 0 && ip - (size_t)ref <= 65535 && load32(src + ref) == seq) {
        size_t p = ip + LZ_MINMATCH, m = (size_t)ref + LZ_MINMATCH;
        while (p < match_end && src[p] == src[m]) {
          p++;
          m++;
        }
        put_sequence(out, src + anchor, ip - anchor, ip - (size_t)ref, p - ip);
        ip = p;
        anchor = p;
      } else {
        ip++;
      }
    }
  }
  put_sequence(out, src + anchor, n - anchor, 0, 0);
}

// Decodes one block into exactly `cap` bytes; false on any malformed input.
bool lz4_decompress(const uint8_t* src, size_t n, uint8_t* dst, size_t cap, size_t* written) {
  size_t ip = 0, op = 0;
  while (ip < n) {
    const uint8_t tok = src[ip++];
    size_t lit = tok >> 4;
    if (lit == 15) {
      uint8_t b;
      do {
        if (ip >= n) return false;
        b = src[ip++];
        lit += b;
      } while (b == 255);
    }
    if (n - ip < lit || cap - op < lit) return false;
    memcpy(dst + op, src + ip, lit);
    ip += lit;
    op += lit;
    if (ip == n) break;  // the last sequence has no match
    if (n - ip < 2) return false;
    const size_t off = (size_t)src[ip] | ((size_t)src[ip + 1] << 8);
    ip += 2;
    if (off == 0 || off > op) return false;
    size_t ml = tok & 15;
    if (ml == 15) {
      uint8_t b;
      do {
        if (ip >= n) return false;
        b = src[ip++];
        ml += b;
      } while (b == 255);
    }
    ml += LZ_MINMATCH;
    if (cap - op < ml) return false;
    for (size_t k = 0; k < ml; k++) dst[op + k] = dst[op - off + k];  // may overlap: byte order
    op += ml;
  }
  *written = op;
  return true;
}

// ---------------------------------------------------------------------------
// JSON (header only).
struct Json {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;
  const Json* get(const char* key) const {
    if (kind != OBJ) return nullptr;
    for (const auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
};

struct JsonParser {
  const char* p;
  const char* end;
  int depth = 0;
  void ws() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
  }
  bool lit(const char* s) {
    const size_t k = strlen(s);
    if ((size_t)(end - p) < k || memcmp(p, s, k) != 0) return false;
    p += k;
    return true;
  }
  static void utf8(std::string& out, uint32_t c) {
    if (c < 0x80) {
      out.push_back((char)c);
    } else if (c < 0x800) {
      out.push_back((char)(0xC0 | (c >> 6)));
      out.push_back((char)(0x80 | (c & 0x3F)));
    } else if (c < 0x10000) {
      out.push_back((char)(0xE0 | (c >> 12)));
      out.push_back((char)(0x80 | ((c >> 6) & 0x3F)));
      out.push_back((char)(0x80 | (c & 0x3F)));
    } else {
      out.push_back((char)(0xF0 | (c >> 18)));
      out.push_back((char)(0x80 | ((c >> 12) & 0x3F)));
      out.push_back((char)(0x80 | ((c >> 6) & 0x3F)));
      out.push_back((char)(0x80 | (c & 0x3F)));
    }
  }
  bool hex4(uint32_t& v) {
    if (end - p < 4) return false;
    v = 0;
    for (int i = 0; i < 4; i++) {
      const char c = *p++;
      v <<= 4;
      if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
      else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
      else return false;
    }
    return true;
  }
  bool string(std::string& out) {
    if (p >= end || *p != '"') return false;
    p++;
    while (p < end && *p != '"') {
      if (*p != '\\') {
        out.push_back(*p++);
        continue;
      }
      if (++p >= end) return false;
      const char e = *p++;
      switch (e) {
        case '"': out.push_back('"'); break;
        case '\\': out.push_back('\\'); break;
        case '/': out.push_back('/'); break;
        case 'b': out.push_back('\b'); break;
        case 'f': out.push_back('\f'); break;
        case 'n': out.push_back('\n'); break;
        case 'r': out.push_back('\r'); break;
        case 't': out.push_back('\t'); break;
        case 'u': {
          uint32_t c;
          if (!hex4(c)) return false;
          if (c >= 0xD800 && c < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
            p += 2;
            uint32_t lo;
            if (!hex4(lo)) return false;
            c = 0x10000 + ((c - 0xD800) << 10) + (lo - 0xDC00);
          }
          utf8(out, c);
          break;
        }
        default: return false;
      }
    }
    if (p >= end) return false;
    p++;
    return true;
  }
  bool value(Json& v) {
    if (++depth > 64) return false;
    ws();
    if (p >= end) return false;
    bool ok = true;
    if (*p == '{') {
      p++;
      v.kind = Json::OBJ;
      ws();
      if (p < end && *p == '}') {
        p++;
      } else {
        for (;;) {
          ws();
          std::string k;
          if (!string(k)) return false;
          ws();
          if (p >= end || *p++ != ':') return false;
          Json child;
          if (!value(child)) return false;
          v.obj.emplace_back(std::move(k), std::move(child));
          ws();
          if (p < end && *p == ',') {
            p++;
            continue;
          }
          if (p < end && *p == '}') {
            p++;
            break;
          }
          return false;
        }
      }
    } else if (*p == '[') {
      p++;
      v.kind = Json::ARR;
      ws();
      if (p < end && *p == ']') {
        p++;
      } else {
        for (;;) {
          Json child;
          if (!value(child)) return false;
          v.arr.push_back(std::move(child));
          ws();
          if (p < end && *p == ',') {
            p++;
            continue;
          }
          if (p < end && *p == ']') {
            p++;
            break;
          }
          return false;
        }
      }
    } else if (*p == '"') {
      v.kind = Json::STR;
      ok = string(v.str);
    } else if (lit("true")) {
      v.kind = Json::BOOL;
      v.b = true;
    } else if (lit("false")) {
      v.kind = Json::BOOL;
      v.b = false;
    } else if (lit("null")) {
      v.kind = Json::NUL;
    } else {
      const char* s = p;
      while (p < end && (strchr("+-.eE", *p) || (*p >= '0' && *p <= '9'))) p++;
      if (p == s) return false;
      const std::string tok(s, p);
      char* stop = nullptr;
      v.kind = Json::NUM;
      v.num = strtod(tok.c_str(), &stop);
      ok = stop && *stop == 0;
    }
    depth--;
    return ok;
  }
};

bool json_number(const Json* v, double& out) {
  if (!v) return false;
  if (v->kind == Json::NUM) {
    out = v->num;
    return true;
  }
  if (v->kind == Json::BOOL) {
    out = v->b ? 1.0 : 0.0;
    return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// SimParams by name (the reference's to_named / set_named: field name, f64
// value; u32 fields as integers).
struct ParamField {
  const char* name;
  size_t offset;
  bool is_float;
};
#define RB_PARAM(f) \
  ParamField { #f, offsetof(ribo_sim_params, f), std::is_same<decltype(ribo_sim_params::f), float>::value }
const ParamField PARAMS[] = {
    RB_PARAM(epoch),
    RB_PARAM(seed),
    RB_PARAM(dt),
    RB_PARAM(diffusion),
    RB_PARAM(settle),
    RB_PARAM(fluid_dt),
    RB_PARAM(fluid_decay),
    RB_PARAM(fluid_vorticity),
    RB_PARAM(fluid_viscosity),
    RB_PARAM(fumarole_count),
    RB_PARAM(uv_strength),
    RB_PARAM(uv_depth),
    RB_PARAM(fluid_enabled),
    RB_PARAM(fluid_obstacle_strength),
    RB_PARAM(slope_steer_rate),
    RB_PARAM(cohesion),
    RB_PARAM(spawn_count),
    RB_PARAM(max_agents),
    RB_PARAM(death_probability),
    RB_PARAM(spawn_energy),
    RB_PARAM(food_power),
    RB_PARAM(maintenance_cost),
    RB_PARAM(pairing_rate),
    RB_PARAM(mutation_rate),
    RB_PARAM(uv_damage),
    RB_PARAM(uptake_rate),
    RB_PARAM(brownian),
    RB_PARAM(phoretic_gain),
    RB_PARAM(chain_stiffness),
    RB_PARAM(thermal_kt),
    RB_PARAM(motor_amplitude),
    RB_PARAM(rft_enabled),
    RB_PARAM(require_start),
    RB_PARAM(joint_coupling),
    RB_PARAM(hunger_regulation),
    RB_PARAM(pairing_cost),
    RB_PARAM(reactivation_rate),
    RB_PARAM(swim_gain),
    RB_PARAM(bioturbation),
    RB_PARAM(bioturbation_cost),
    RB_PARAM(monomer_uv_absorb),
    RB_PARAM(sedimentation),
    RB_PARAM(direct_photoactivation),
    RB_PARAM(activation_decay),
    RB_PARAM(monomer_pressure),
    RB_PARAM(agent_fluid_push),
    RB_PARAM(swim_wobble),
    RB_PARAM(fluid_swim_only),
    RB_PARAM(motion_cost),
    RB_PARAM(bond_rate),
    RB_PARAM(bond_energy_share),
    RB_PARAM(bond_signal),
    RB_PARAM(aggregation),
    RB_PARAM(photo_yield),
    RB_PARAM(heat_kill),
    RB_PARAM(flow_coupling),
    RB_PARAM(inertia),
    RB_PARAM(death_energy_cap),
    RB_PARAM(chemo_yield),
    RB_PARAM(redox_decay),
    RB_PARAM(thermal_activation),
    RB_PARAM(denature_temp),
    RB_PARAM(day_period),
    RB_PARAM(sun_slope),
    RB_PARAM(sun_now),
    RB_PARAM(sun_angle),
    RB_PARAM(day_fraction),
    RB_PARAM(metabolic_q10),
    RB_PARAM(metabolic_span),
    RB_PARAM(metabolic_ref),
    RB_PARAM(sun_heat),
    RB_PARAM(sediment_transport),
    RB_PARAM(sediment_threshold),
    RB_PARAM(sediment_settle),
    RB_PARAM(signal_mode),
    RB_PARAM(clock_mute),
    RB_PARAM(paint_x),
    RB_PARAM(paint_y),
    RB_PARAM(paint_radius),
    RB_PARAM(paint_grains),
    RB_PARAM(rest_angle_mult),
    RB_PARAM(protease_power),
    RB_PARAM(lysis_yield),
    RB_PARAM(protease_direct),
    RB_PARAM(joint_load),
    RB_PARAM(swim_grip),
    RB_PARAM(swim_memory),
    RB_PARAM(mouth_leak),
    RB_PARAM(leak_base),
    RB_PARAM(skin_uptake),
    RB_PARAM(death_metab),
    RB_PARAM(salvage),
    RB_PARAM(bond_matter_share),
    RB_PARAM(brownian_rot),
    RB_PARAM(transport_every),
    RB_PARAM(signal_crosstalk),
    RB_PARAM(flow_mass),
    RB_PARAM(chemo_take),
    RB_PARAM(vent_cycle_period),
    RB_PARAM(vent_cycle_amp),
    RB_PARAM(sediment_cohesion),
    RB_PARAM(sediment_compaction),
    RB_PARAM(rock_crumble),
    RB_PARAM(lysis_matter),
    RB_PARAM(scramble_conduction),
    RB_PARAM(scramble_angles),
    RB_PARAM(scramble_response),
    RB_PARAM(scramble_amount),
    RB_PARAM(pairing_energy_half),
    RB_PARAM(pairing_min_energy),
    RB_PARAM(uv_mutation),
    RB_PARAM(heat_mutation),
    RB_PARAM(birth_crowding),
    RB_PARAM(photo_damage),
    RB_PARAM(naked_decay),
    RB_PARAM(store_loss),
};
#undef RB_PARAM
constexpr size_t NPARAMS = sizeof(PARAMS) / sizeof(PARAMS[0]);
static_assert(NPARAMS * 4 == sizeof(ribo_sim_params), "every SimParams field is named");

void json_escape(std::string& out, const char* s) {
  out.push_back('"');
  for (; *s; s++) {
    const unsigned char c = (unsigned char)*s;
    if (c == '"' || c == '\\') {
      out.push_back('\\');
      out.push_back((char)c);
    } else if (c < 0x20) {
      char buf[8];
      snprintf(buf, sizeof buf, "\\u%04x", c);
      out += buf;
    } else {
      out.push_back((char)c);
    }
  }
  out.push_back('"');
}
void json_key(std::string& out, const char* k, bool& first) {
  if (!first) out += ",\n    ";
  first = false;
  json_escape(out, k);
  out += ": ";
}
std::string fmt_num(double v) {
  char buf[40];
  snprintf(buf, sizeof buf, "%.17g", v);
  return buf;
}

// ---------------------------------------------------------------------------
// The container.
const char MAGIC[8] = {'R', 'I', 'B', 'O', 'S', 'C', 'N', '1'};
// The reference's agent blocks, written empty (zero agents).
const char* const AGENT_BLOCKS[] = {"agents",      "genomes",    "bodies",     "organs",       "rna_tails4",
                                    "bitten",      "body_pos",   "signals4",   "joint_angle",  "joint_base",
                                    "joint_state", "joint_active", "sensor_mem", "bonds2",     "pair_mask"};

void put_u16(std::vector<uint8_t>& out, uint16_t v) {
  out.push_back((uint8_t)(v & 0xff));
  out.push_back((uint8_t)(v >> 8));
}
void put_u32(std::vector<uint8_t>& out, uint32_t v) {
  for (int i = 0; i < 4; i++) out.push_back((uint8_t)(v >> (8 * i)));
}
void put_u64(std::vector<uint8_t>& out, uint64_t v) {
  for (int i = 0; i < 8; i++) out.push_back((uint8_t)(v >> (8 * i)));
}
uint64_t get_le(const uint8_t* p, int n) {
  uint64_t v = 0;
  for (int i = 0; i < n; i++) v |= (uint64_t)p[i] << (8 * i);
  return v;
}

void put_block(std::vector<uint8_t>& out, const char* name, const void* data, size_t n) {
  std::vector<uint8_t> c;
  lz4_compress(static_cast<const uint8_t*>(data), n, c);
  const size_t nl = strlen(name);
  put_u16(out, (uint16_t)nl);
  out.insert(out.end(), name, name + nl);
  put_u64(out, (uint64_t)c.size() + 4);
  put_u32(out, (uint32_t)n);
  out.insert(out.end(), c.begin(), c.end());
}

struct SceneBlocks {
  std::vector<std::pair<std::string, std::vector<uint8_t>>> blocks;
  const std::vector<uint8_t>* find(const char* name) const {
    for (const auto& b : blocks)
      if (b.first == name) return &b.second;
    return nullptr;
  }
};

ribo_status parse_scene(const std::vector<uint8_t>& bytes, Json& header, SceneBlocks& out) {
  if (bytes.size() < 12 || memcmp(bytes.data(), MAGIC, 8) != 0)
    return set_error(RIBO_INVALID_ARG, "not a ribossome scene (magic)");
  const size_t hl = (size_t)get_le(bytes.data() + 8, 4);
  if (hl > bytes.size() - 12) return set_error(RIBO_INVALID_ARG, "scene header runs past the file");
  JsonParser jp{reinterpret_cast<const char*>(bytes.data()) + 12, reinterpret_cast<const char*>(bytes.data()) + 12 + hl};
  if (!jp.value(header) || header.kind != Json::OBJ) return set_error(RIBO_INVALID_ARG, "scene header: malformed JSON");
  size_t p = 12 + hl;
  while (p < bytes.size()) {
    if (bytes.size() - p < 2) return set_error(RIBO_INVALID_ARG, "scene block: truncated name length");
    const size_t nl = (size_t)get_le(bytes.data() + p, 2);
    p += 2;
    if (bytes.size() - p < nl + 8) return set_error(RIBO_INVALID_ARG, "scene block: truncated");
    std::string name(reinterpret_cast<const char*>(bytes.data()) + p, nl);
    p += nl;
    const uint64_t cl = get_le(bytes.data() + p, 8);
    p += 8;
    if (cl < 4 || cl > bytes.size() - p) return set_error(RIBO_INVALID_ARG, "scene block %s: bad length", name.c_str());
    const size_t raw = (size_t)get_le(bytes.data() + p, 4);
    std::vector<uint8_t> data(raw);
    size_t got = 0;
    if (!lz4_decompress(bytes.data() + p + 4, (size_t)cl - 4, data.data(), raw, &got) || got != raw)
      return set_error(RIBO_INVALID_ARG, "scene block %s: corrupt LZ4 data", name.c_str());
    p += (size_t)cl;
    out.blocks.emplace_back(std::move(name), std::move(data));
  }
  return RIBO_OK;
}

bool read_file(const char* path, std::vector<uint8_t>& out) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  uint8_t buf[1 << 16];
  size_t k;
  while ((k = fread(buf, 1, sizeof buf, f)) > 0) out.insert(out.end(), buf, buf + k);
  const bool ok = !ferror(f);
  fclose(f);
  return ok;
}

// Settings of this path in the header ("gb300_settings"), and the
// reference's own keys ("settings", src/world/mod.rs:92-115).
struct SettingField {
  const char* name;
  size_t offset;
  bool is_float;
};
#define RB_SETTING(f) \
  SettingField { #f, offsetof(ribo_world_settings, f), std::is_same<decltype(ribo_world_settings::f), float>::value }
const SettingField SETTINGS[] = {RB_SETTING(fluid_enabled),  RB_SETTING(fluid_substep),   RB_SETTING(multigrid),
                                 RB_SETTING(mg_cycles),      RB_SETTING(jacobi_iters),    RB_SETTING(ledger_each_step),
                                 RB_SETTING(mg_unfused),     RB_SETTING(transport_simple), RB_SETTING(mixed_tol),
                                 RB_SETTING(mixed_inner_tol), RB_SETTING(mixed_max_outer), RB_SETTING(mixed_max_inner),
                                 RB_SETTING(mixed_alpha),    RB_SETTING(light_mode),      RB_SETTING(light_rows_per_step),
                                 RB_SETTING(light_interval), RB_SETTING(terrain_mode)};
#undef RB_SETTING
static_assert(sizeof(SETTINGS) / sizeof(SETTINGS[0]) * 4 == sizeof(ribo_world_settings), "every setting is named");

}  // namespace
}  // namespace ribo

using namespace ribo;

extern "C" const char* ribo_sim_param_name(uint32_t i) { return i < NPARAMS ? PARAMS[i].name : nullptr; }

extern "C" size_t ribo_lz4_compress_bound(size_t n) { return n + n / 255 + 16; }

extern "C" ribo_status ribo_lz4_compress(const void* src, size_t n, void* dst, size_t cap, size_t* written) {
  if ((!src && n) || !dst || !written) return set_error(RIBO_INVALID_ARG, "null argument");
  std::vector<uint8_t> c;
  lz4_compress(static_cast<const uint8_t*>(src), n, c);
  if (c.size() > cap) return set_error(RIBO_INVALID_ARG, "output buffer too small (%zu < %zu)", cap, c.size());
  memcpy(dst, c.data(), c.size());
  *written = c.size();
  return RIBO_OK;
}

extern "C" ribo_status ribo_lz4_decompress(const void* src, size_t n, void* dst, size_t cap, size_t* written) {
  if ((!src && n) || (!dst && cap) || !written) return set_error(RIBO_INVALID_ARG, "null argument");
  size_t got = 0;
  if (!lz4_decompress(static_cast<const uint8_t*>(src), n, static_cast<uint8_t*>(dst), cap, &got))
    return set_error(RIBO_INVALID_ARG, "malformed LZ4 block or output buffer too small");
  *written = got;
  return RIBO_OK;
}

extern "C" ribo_status ribo_world_save_scene(ribo_world* w, const char* path, const ribo_sim_params* params) {
  if (!w || !path || !params) return set_error(RIBO_INVALID_ARG, "null argument");
  const World& W = w->w;
  const ribo_world_cfg& c = W.cfg;
  struct Field {
    const char* name;
    ribo_field f;
  };
  const Field fields[] = {{"chem", RIBO_FIELD_CHEM},         {"gamma", RIBO_FIELD_GAMMA},
                         {"velocity", RIBO_FIELD_VELOCITY}, {"pressure", RIBO_FIELD_PRESSURE},
                         {"temperature", RIBO_FIELD_TEMP},  {"redox", RIBO_FIELD_REDOX},
                         {"gb300_heat", RIBO_FIELD_HEAT},   {"gb300_light", RIBO_FIELD_LIGHT},
                         {"gb300_shade", RIBO_FIELD_SHADE}};
  std::vector<std::vector<uint8_t>> data;
  for (const Field& f : fields) {
    data.emplace_back(field_bytes_of(c, f.f));
    ribo_status st = ribo_world_read(w, f.f, data.back().data(), data.back().size());
    if (st != RIBO_OK) return st;
  }
  // header (the reference's keys; "gb300_settings" and grid_w/grid_h are ours)
  std::string h = "{\n    ";
  bool first = true;
  json_key(h, "versao", first);
  h += "2";
  json_key(h, "gravado", first);
  h += fmt_num((double)time(nullptr));
  json_key(h, "agentes", first);
  h += "0";
  json_key(h, "cfg", first);
  h += "{\"grid_size\": " + fmt_num(c.grid_w) + ", \"fluid_size\": " + fmt_num(c.fluid_w) +
       ", \"world_units_per_cell\": " + fmt_num(c.world_units_per_cell) + ", \"max_agents\": 0, \"grid_w\": " +
       fmt_num(c.grid_w) + ", \"grid_h\": " + fmt_num(c.grid_h) + ", \"fluid_w\": " + fmt_num(c.fluid_w) +
       ", \"fluid_h\": " + fmt_num(c.fluid_h) + "}";
  json_key(h, "params", first);
  h += "{";
  for (size_t i = 0; i < NPARAMS; i++) {
    if (i) h += ", ";
    json_escape(h, PARAMS[i].name);
    h += ": ";
    const uint8_t* base = reinterpret_cast<const uint8_t*>(params) + PARAMS[i].offset;
    if (PARAMS[i].is_float) {
      float v;
      memcpy(&v, base, 4);
      h += fmt_num((double)v);
    } else {
      uint32_t v;
      memcpy(&v, base, 4);
      h += fmt_num((double)v);
    }
  }
  h += "}";
  const ribo_world_settings& s = W.st;
  json_key(h, "settings", first);
  h += std::string("{\"fluid_enabled\": ") + (s.fluid_enabled ? "true" : "false") +
       ", \"fluid_substep\": " + fmt_num(s.fluid_substep) + ", \"multigrid\": " + (s.multigrid ? "true" : "false") +
       ", \"mg_cycles\": " + fmt_num(s.mg_cycles) + ", \"jacobi_iters\": " + fmt_num(s.jacobi_iters) +
       ", \"light_rows_per_step\": " + fmt_num(s.light_rows_per_step) + ", \"light_interval\": " +
       fmt_num(s.light_interval) + ", \"terrain_enabled\": false, \"contact_enabled\": true}";
  json_key(h, "gb300_settings", first);
  h += "{";
  for (size_t i = 0; i < sizeof(SETTINGS) / sizeof(SETTINGS[0]); i++) {
    if (i) h += ", ";
    json_escape(h, SETTINGS[i].name);
    h += ": ";
    const uint8_t* base = reinterpret_cast<const uint8_t*>(&s) + SETTINGS[i].offset;
    if (SETTINGS[i].is_float) {
      float v;
      memcpy(&v, base, 4);
      h += fmt_num((double)v);
    } else {
      uint32_t v;
      memcpy(&v, base, 4);
      h += fmt_num((double)v);
    }
  }
  h += "}";
  json_key(h, "fumarolas", first);
  h += "[]";
  json_key(h, "interface", first);
  h += "{}";
  h += "\n}";

  std::vector<uint8_t> out(MAGIC, MAGIC + 8);
  put_u32(out, (uint32_t)h.size());
  out.insert(out.end(), h.begin(), h.end());
  put_block(out, "slots", nullptr, 0);
  const uint32_t counters[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  put_block(out, "life_counters", counters, sizeof counters);
  for (const char* name : AGENT_BLOCKS) put_block(out, name, nullptr, 0);
  for (size_t i = 0; i < sizeof(fields) / sizeof(fields[0]); i++)
    put_block(out, fields[i].name, data[i].data(), data[i].size());

  // written to a temporary file first, then renamed over the target
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = fopen(tmp.c_str(), "wb");
  if (!f) return set_error(RIBO_INVALID_ARG, "cannot write %s", tmp.c_str());
  const bool ok = fwrite(out.data(), 1, out.size(), f) == out.size();
  if (fclose(f) != 0 || !ok) {
    remove(tmp.c_str());
    return set_error(RIBO_INVALID_ARG, "write to %s failed", tmp.c_str());
  }
  if (rename(tmp.c_str(), path) != 0) {
    remove(tmp.c_str());
    return set_error(RIBO_INVALID_ARG, "cannot rename %s to %s", tmp.c_str(), path);
  }
  return RIBO_OK;
}

extern "C" ribo_status ribo_world_load_scene(ribo_world* w, const char* path, ribo_sim_params* params) {
  if (!w || !path) return set_error(RIBO_INVALID_ARG, "null argument");
  std::vector<uint8_t> bytes;
  if (!read_file(path, bytes)) return set_error(RIBO_INVALID_ARG, "cannot read %s", path);
  Json header;
  SceneBlocks blocks;
  ribo_status st = parse_scene(bytes, header, blocks);
  if (st != RIBO_OK) return st;
  World& W = w->w;
  const ribo_world_cfg& c = W.cfg;
  // sizes must match (src/world/snapshot.rs:391-397)
  const Json* cfg = header.get("cfg");
  double gs = 0, fs = 0, upc = 0, gw = 0, gh = 0, fw = 0, fh = 0;
  if (!cfg || !json_number(cfg->get("grid_size"), gs) || !json_number(cfg->get("fluid_size"), fs) ||
      !json_number(cfg->get("world_units_per_cell"), upc))
    return set_error(RIBO_INVALID_ARG, "scene header: cfg missing");
  if (!json_number(cfg->get("grid_w"), gw)) gw = gs;
  if (!json_number(cfg->get("grid_h"), gh)) gh = gs;
  if (!json_number(cfg->get("fluid_w"), fw)) fw = fs;
  if (!json_number(cfg->get("fluid_h"), fh)) fh = fs;
  if (gw != c.grid_w || gh != c.grid_h || fw != c.fluid_w || fh != c.fluid_h || upc != c.world_units_per_cell)
    return set_error(RIBO_INVALID_ARG, "the scene is from another world size (%gx%g, fluid %gx%g, %g units/cell)", gw, gh,
                     fw, fh, upc);
  // every world block present with its exact size before anything changes
  struct Field {
    const char* name;
    ribo_field f;
    bool required;
  };
  const Field fields[] = {{"gamma", RIBO_FIELD_GAMMA, true},         {"chem", RIBO_FIELD_CHEM, true},
                          {"velocity", RIBO_FIELD_VELOCITY, true},   {"pressure", RIBO_FIELD_PRESSURE, true},
                          {"temperature", RIBO_FIELD_TEMP, true},    {"redox", RIBO_FIELD_REDOX, false},
                          {"gb300_heat", RIBO_FIELD_HEAT, false},    {"gb300_light", RIBO_FIELD_LIGHT, false},
                          {"gb300_shade", RIBO_FIELD_SHADE, false}};
  for (const Field& f : fields) {
    const std::vector<uint8_t>* b = blocks.find(f.name);
    if (!b) {
      if (f.required) return set_error(RIBO_INVALID_ARG, "scene block %s is missing", f.name);
      continue;
    }
    if (b->size() != field_bytes_of(c, f.f))
      return set_error(RIBO_INVALID_ARG, "scene block %s has the wrong size (%zu bytes)", f.name, b->size());
  }
  // parameters by name over the defaults (src/world/snapshot.rs:414-427)
  ribo_sim_params p;
  ribo_sim_params_default(&p);
  if (const Json* named = header.get("params")) {
    if (named->kind == Json::OBJ)
      for (const auto& kv : named->obj) {
        double v;
        if (!json_number(&kv.second, v)) continue;
        for (size_t i = 0; i < NPARAMS; i++) {
          if (kv.first != PARAMS[i].name) continue;
          uint8_t* base = reinterpret_cast<uint8_t*>(&p) + PARAMS[i].offset;
          if (PARAMS[i].is_float) {
            const float f = (float)v;
            memcpy(base, &f, 4);
          } else {
            const uint32_t u = v <= 0.0 ? 0u : v >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)v;
            memcpy(base, &u, 4);
          }
          break;
        }
      }
  }
  // settings: the reference's keys, then this path's own when present
  ribo_world_settings s = W.st;
  if (const Json* rs = header.get("settings")) {
    double v;
    if (json_number(rs->get("fluid_enabled"), v)) s.fluid_enabled = v != 0.0;
    if (json_number(rs->get("fluid_substep"), v)) s.fluid_substep = (uint32_t)v;
    if (json_number(rs->get("multigrid"), v)) s.multigrid = v != 0.0;
    if (json_number(rs->get("mg_cycles"), v)) s.mg_cycles = (uint32_t)v;
    if (json_number(rs->get("jacobi_iters"), v)) s.jacobi_iters = (uint32_t)v;
    if (json_number(rs->get("light_rows_per_step"), v)) s.light_rows_per_step = (uint32_t)v;
    if (json_number(rs->get("light_interval"), v)) s.light_interval = (uint32_t)v;
  }
  if (const Json* gs8 = header.get("gb300_settings")) {
    for (const SettingField& f : SETTINGS) {
      double v;
      if (!json_number(gs8->get(f.name), v)) continue;
      uint8_t* base = reinterpret_cast<uint8_t*>(&s) + f.offset;
      if (f.is_float) {
        const float x = (float)v;
        memcpy(base, &x, 4);
      } else {
        const uint32_t x = v <= 0.0 ? 0u : (uint32_t)v;
        memcpy(base, &x, 4);
      }
    }
  }
  if ((st = ribo_world_set_settings(w, &s)) != RIBO_OK) return st;
  for (const Field& f : fields) {
    const std::vector<uint8_t>* b = blocks.find(f.name);
    if (!b) continue;
    if ((st = ribo_world_upload(w, f.f, b->data(), b->size())) != RIBO_OK) return st;
  }
  if (params) *params = p;
  return ribo_world_sync(w);
}

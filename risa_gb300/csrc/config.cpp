// Reader for the reference's configuration files (RISA/example/config.cfg),
// which are libconfig documents: `key = value;` settings with numbers,
// strings, booleans, arrays `[ ... ]` and lists `( ... )`, and //, # and
// /* */ comments. The reference reads them through libconfig++
// (ConfigReader.h:62-86) and each stage's readConfig picks its own keys; a
// parse error there ends the process (ConfigReader.cpp:35-41). This reader
// returns RISA_GB_ECONFIG with a message instead.
#include "risa_gb_internal.h"

#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>

namespace risa_gb {

namespace {
struct Value {
   enum Kind { kNumber, kString, kBool, kArray, kOther } kind = kOther;
   double num = 0.0;
   bool is_int = false;
   long long inum = 0;
   std::string str;
   std::vector<Value> items;
};

struct Parser {
   std::string s;
   size_t i = 0;
   int line = 1;
   std::string err;

   void skip_ws() {
      while (i < s.size()) {
         const char c = s[i];
         if (c == '\n') { ++line; ++i; }
         else if (std::isspace((unsigned char)c)) ++i;
         else if (c == '#' || (c == '/' && i + 1 < s.size() && s[i + 1] == '/')) {
            while (i < s.size() && s[i] != '\n') ++i;
         } else if (c == '/' && i + 1 < s.size() && s[i + 1] == '*') {
            i += 2;
            while (i + 1 < s.size() && !(s[i] == '*' && s[i + 1] == '/')) {
               if (s[i] == '\n') ++line;
               ++i;
            }
            i += 2;
         } else break;
      }
   }
   bool ident(std::string* out) {
      skip_ws();
      const size_t b = i;
      while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' || s[i] == '*')) ++i;
      *out = s.substr(b, i - b);
      return !out->empty();
   }
   bool value(Value* v) {
      skip_ws();
      if (i >= s.size()) { err = "unexpected end of file"; return false; }
      const char c = s[i];
      if (c == '"') {
         ++i;
         std::string str;
         while (i < s.size() && s[i] != '"') {
            if (s[i] == '\\' && i + 1 < s.size()) ++i;
            str += s[i++];
         }
         if (i >= s.size()) { err = "unterminated string"; return false; }
         ++i;
         v->kind = Value::kString;
         v->str = str;
         skip_ws();
         while (i < s.size() && s[i] == '"') {  // adjacent strings concatenate
            Value more;
            if (!value(&more)) return false;
            v->str += more.str;
         }
         return true;
      }
      if (c == '[' || c == '(') {
         const char close = c == '[' ? ']' : ')';
         ++i;
         v->kind = c == '[' ? Value::kArray : Value::kOther;
         skip_ws();
         if (i < s.size() && s[i] == close) { ++i; return true; }
         while (true) {
            Value item;
            if (!value(&item)) return false;
            v->items.push_back(item);
            skip_ws();
            if (i < s.size() && s[i] == ',') { ++i; continue; }
            if (i < s.size() && s[i] == close) { ++i; return true; }
            err = "expected ',' or closing bracket";
            return false;
         }
      }
      if (c == '{') {  // group: skip balanced braces
         int depth = 0;
         do {
            if (s[i] == '{') ++depth;
            if (s[i] == '}') --depth;
            if (s[i] == '\n') ++line;
            ++i;
         } while (i < s.size() && depth > 0);
         v->kind = Value::kOther;
         return true;
      }
      const size_t b = i;
      while (i < s.size() && !std::isspace((unsigned char)s[i]) && s[i] != ';' && s[i] != ',' &&
             s[i] != ']' && s[i] != ')')
         ++i;
      const std::string tok = s.substr(b, i - b);
      if (tok == "true" || tok == "TRUE" || tok == "false" || tok == "FALSE") {
         v->kind = Value::kBool;
         v->num = (tok[0] == 't' || tok[0] == 'T') ? 1.0 : 0.0;
         return true;
      }
      char* end = nullptr;
      std::string t = tok;
      if (!t.empty() && (t.back() == 'L')) t.pop_back();
      if (!t.empty() && (t.back() == 'L')) t.pop_back();
      const bool looks_int = t.find_first_of(".eE") == std::string::npos ||
                             (t.size() > 2 && (t[1] == 'x' || t[1] == 'X'));
      if (looks_int) {
         const long long iv = std::strtoll(t.c_str(), &end, 0);
         if (end && *end == '\0' && !t.empty()) {
            v->kind = Value::kNumber;
            v->is_int = true;
            v->inum = iv;
            v->num = (double)iv;
            return true;
         }
      }
      const double dv = std::strtod(t.c_str(), &end);
      if (end && *end == '\0' && !t.empty()) {
         v->kind = Value::kNumber;
         v->num = dv;
         return true;
      }
      err = "cannot parse value '" + tok + "'";
      return false;
   }
   bool parse(std::map<std::string, Value>* out) {
      while (true) {
         skip_ws();
         if (i >= s.size()) return true;
         std::string key;
         if (!ident(&key)) { err = "expected a setting name"; return false; }
         skip_ws();
         if (i < s.size() && (s[i] == '=' || s[i] == ':')) ++i;
         else { err = "expected '=' after " + key; return false; }
         Value v;
         if (!value(&v)) return false;
         (*out)[key] = v;
         skip_ws();
         if (i < s.size() && (s[i] == ';' || s[i] == ',')) ++i;
      }
   }
};
}  // namespace

namespace {
risa_gb_status parse_file(const char* path, std::map<std::string, Value>* kv) {
   std::ifstream in(path);
   if (!in) return fail(RISA_GB_ECONFIG, std::string("config: cannot open ") + path);
   std::stringstream ss;
   ss << in.rdbuf();
   Parser ps;
   ps.s = ss.str();
   if (!ps.parse(kv))
      return fail(RISA_GB_ECONFIG, std::string("config: parse error at ") + path + ":" +
                                       std::to_string(ps.line) + " - " + ps.err);
   return RISA_GB_OK;
}

std::string to_text(const Value& v) {
   switch (v.kind) {
      case Value::kString: return v.str;
      case Value::kBool: return v.num != 0.0 ? "true" : "false";
      case Value::kNumber: {
         if (v.is_int) return std::to_string(v.inum);
         std::ostringstream os;
         os.precision(17);
         os << v.num;
         return os.str();
      }
      case Value::kArray: {
         std::string out;
         for (size_t i = 0; i < v.items.size(); ++i) out += (i ? "," : "") + to_text(v.items[i]);
         return out;
      }
      default: return "";
   }
}
}  // namespace

risa_gb_status lookup_config(const char* path, const char* key, char* value, size_t value_len) {
   if (!path || !key || !value || value_len == 0) return fail(RISA_GB_EINVAL, "config: null argument");
   std::map<std::string, Value> kv;
   risa_gb_status st = parse_file(path, &kv);
   if (st) return st;
   auto it = kv.find(key);
   if (it == kv.end()) return fail(RISA_GB_ECONFIG, std::string("config: no setting ") + key);
   const std::string text = to_text(it->second);
   if (text.size() + 1 > value_len) return fail(RISA_GB_EINVAL, "config: value buffer too small");
   std::memcpy(value, text.c_str(), text.size() + 1);
   return RISA_GB_OK;
}

risa_gb_status load_config(const char* path, risa_gb_geometry* g, risa_gb_params* p) {
   if (!path || !g || !p) return fail(RISA_GB_EINVAL, "config: null argument");
   std::map<std::string, Value> kv;
   risa_gb_status pst = parse_file(path, &kv);
   if (pst) return pst;
   risa_gb_geometry_init(g);
   risa_gb_params_init(p);
   auto num = [&](const char* k, double* out) {
      auto it = kv.find(k);
      if (it == kv.end() || (it->second.kind != Value::kNumber && it->second.kind != Value::kBool))
         return false;
      *out = it->second.num;
      return true;
   };
   auto inum = [&](const char* k, int32_t* out) {
      double d;
      if (!num(k, &d)) return false;
      *out = (int32_t)d;
      return true;
   };
   auto str = [&](const char* k, std::string* out) {
      auto it = kv.find(k);
      if (it == kv.end() || it->second.kind != Value::kString) return false;
      *out = it->second.str;
      return true;
   };
   auto arr = [&](const char* k, double* out) {
      auto it = kv.find(k);
      if (it == kv.end()) return false;
      if (it->second.kind == Value::kNumber) {
         for (int j = 0; j < RISA_GB_MAX_PLANES; ++j) out[j] = it->second.num;
         return true;
      }
      if (it->second.kind != Value::kArray || it->second.items.empty()) return false;
      for (int j = 0; j < RISA_GB_MAX_PLANES; ++j) {
         const auto& items = it->second.items;
         out[j] = items[j < (int)items.size() ? j : items.size() - 1].num;
      }
      return true;
   };
   // Required keys: the union of what the hot-path stages read
   // (Attenuation.cu:387-408, Fan2Para.cu:595-619, Filter.cu:196-201,
   // Backprojection.cu:214-222).
   int32_t sampling = 0, scan = 0;
   std::string missing;
   auto need = [&](bool ok, const char* k) {
      if (!ok) missing += std::string(missing.empty() ? "" : ", ") + k;
   };
   need(inum("numberOfFanDetectors", &g->n_fan_det), "numberOfFanDetectors");
   need(inum("samplingRate", &sampling), "samplingRate");
   need(inum("scanRate", &scan), "scanRate");
   need(inum("numberOfParallelProjections", &g->n_par_proj), "numberOfParallelProjections");
   need(inum("numberOfParallelDetectors", &g->n_par_det), "numberOfParallelDetectors");
   need(inum("numberOfPixels", &g->n_pixels), "numberOfPixels");
   need(num("detectorDiameter", &g->detector_diameter), "detectorDiameter");
   need(num("imageWidth", &g->image_width), "imageWidth");
   need(arr("sourceDiameter", g->source_diameter), "sourceDiameter");
   if (!missing.empty()) return fail(RISA_GB_ECONFIG, "config: missing " + missing);
   if (scan <= 0) return fail(RISA_GB_ECONFIG, "config: scanRate must be positive");
   g->n_fan_proj = (int32_t)((long long)sampling * 1000000LL / scan);
   inum("numberOfPlanes", &g->n_planes);
   inum("numberOfDetectorModules", &g->n_modules);
   num("sourceOffset", &g->source_offset);
   num("imageCenterX", &g->image_center_x);
   num("imageCenterY", &g->image_center_y);
   num("rotationOffset", &g->rotation_offset);
   arr("deltaX", g->delta_x);
   arr("deltaZ", g->delta_z);
   arr("sourceAngle", g->source_angle);

   std::string s;
   if (str("filterType", &s)) {
      // Filter.cu:202-215: unknown names fall back to ramp
      if (s == "sheppLogan") p->filter_type = RISA_GB_FILTER_SHEPP_LOGAN;
      else if (s == "hamming") p->filter_type = RISA_GB_FILTER_HAMMING;
      else if (s == "hanning") p->filter_type = RISA_GB_FILTER_HANNING;
      else if (s == "cosine") p->filter_type = RISA_GB_FILTER_COSINE;
      else p->filter_type = RISA_GB_FILTER_RAMP;
   }
   num("cutoffFraction", &p->cutoff);
   if (str("interpolationType", &s))
      p->interp = (s == "nearestNeighbour") ? RISA_GB_INTERP_NEAREST : RISA_GB_INTERP_LINEAR;
   double d = 0;
   if (num("useTextureMemory", &d) && d != 0.0) p->interp = RISA_GB_INTERP_NEAREST_TRUNC;
   num("thresh_min", &p->thresh_min);
   num("thresh_max", &p->thresh_max);
   num("lowerLimOffset", &p->lower_lim_offset);
   num("upperLimOffset", &p->upper_lim_offset);
   int32_t xv;
   if (inum("xa", &xv)) p->xa = (uint32_t)xv;
   if (inum("xb", &xv)) p->xb = (uint32_t)xv;
   if (inum("xc", &xv)) p->xc = (uint32_t)xv;
   if (inum("xd", &xv)) p->xd = (uint32_t)xv;
   if (inum("xe", &xv)) p->xe = (uint32_t)xv;
   if (inum("xf", &xv)) p->xf = (uint32_t)xv;
   if (num("normalization", &d)) p->normalize = d != 0.0;
   num("maskingValue", &p->masking_value);
   // this library's own keys
   if (str("gb_quirks", &s)) {
      if (s == "risa") p->quirks = RISA_GB_QUIRKS_RISA;
      else if (s == "none") p->quirks = RISA_GB_QUIRKS_NONE;
      else return fail(RISA_GB_ECONFIG, "config: gb_quirks must be \"risa\" or \"none\"");
   }
   inum("gb_pad", &p->pad);
   if (num("gb_defects", &d)) p->defects = d != 0.0;
   if (num("gb_relevant_mask", &d)) p->relevant_mask = d != 0.0;
   if (num("gb_masking", &d)) p->masking = d != 0.0;
   if (num("gb_repair_reference", &d)) p->repair_reference = d != 0.0;
   if (num("gb_module_major", &d)) p->module_major = d != 0.0;
   return RISA_GB_OK;
}

}  // namespace risa_gb

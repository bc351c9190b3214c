// Minimal stand-in for libconfig++ (not installed). The harness never parses a
// file through it: it only has to satisfy the declarations the reference's
// ConfigReader header uses.
#pragma once
#include <string>
namespace libconfig {
struct Setting {
   int getLength() const { return 0; }
   const Setting& operator[](int) const { return *this; }
   operator float() const { return 0.f; }
   operator double() const { return 0.0; }
   operator int() const { return 0; }
};
struct FileIOException {};
struct ParseException {
   const char* getFile() const { return ""; }
   int getLine() const { return 0; }
   const char* getError() const { return ""; }
};
class Config {
 public:
   void readFile(const char*) {}
   template <typename T> bool lookupValue(const char*, T&) const { return false; }
   Setting& lookup(const char*) { static Setting s; return s; }
};
}

// tsplib.cu -- TSPLIB .tsp reader of the C ABI (aco_tsplib_*), host code.
//
// Restates TSPReader::read (src/TSPReader.cu:25-95): lines of one character or
// less are skipped; a trailing non-printable character (a CR) is dropped;
// "TAG : value" is split at the first ':' and every space is removed from
// both sides; TYPE must be TSP or STSP and EDGE_WEIGHT_TYPE must be EUC_2D;
// DIMENSION gives the node count; NODE_COORD_SECTION is followed by that many
// "id x y" lines read with "%ld %f %f"; an EOF line ends the file.  Where the
// reference reads past what the file holds (a coordinate section before
// DIMENSION, a short or unparsable coordinate line, too few lines) it leaves
// values uninitialised; here those files are rejected with ACO_ERR_FORMAT.
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>

#include <fstream>
#include <new>
#include <string>
#include <vector>

#include "acogpu.h"

struct aco_tsplib {
  std::string name;
  std::vector<float> x, y;
};

namespace {

thread_local std::string g_tsplib_error;

int tsplib_fail(int status, const std::string &msg) {
  g_tsplib_error = msg;
  return status;
}

void strip_trailing_unprintable(std::string &line) {
  if (!line.empty() && !isprint(static_cast<unsigned char>(line.back()))) line.pop_back();
}

void remove_spaces(std::string &s) {
  std::string out;
  out.reserve(s.size());
  for (char ch : s)
    if (ch != ' ') out.push_back(ch);
  s.swap(out);
}

}  // namespace

extern "C" {

int aco_tsplib_read(const char *path, aco_tsplib **out) {
  if (!path || !out) return tsplib_fail(ACO_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  std::ifstream in(path, std::ios_base::in);
  if (!in) return tsplib_fail(ACO_ERR_IO, std::string("unable to open file: ") + path);
  aco_tsplib *t = new (std::nothrow) aco_tsplib();
  if (!t) return tsplib_fail(ACO_ERR_OUT_OF_MEMORY, "out of memory");
  long nodes = -1;
  bool have_coords = false;
  std::string line;
  while (in.good()) {
    std::getline(in, line);
    if (line.length() <= 1) continue;
    strip_trailing_unprintable(line);
    std::string tag, value;
    const size_t colon = line.find(':');
    if (colon != std::string::npos) {
      tag = line.substr(0, colon);
      value = line.substr(colon + 1);
    } else {
      tag = line;
    }
    remove_spaces(tag);
    remove_spaces(value);
    if (tag == "NAME") {
      t->name = value;
    } else if (tag == "TYPE") {
      if (value != "TSP" && value != "STSP") {
        delete t;
        return tsplib_fail(ACO_ERR_FORMAT, "invalid problem type: " + value);
      }
    } else if (tag == "DIMENSION") {
      nodes = atol(value.c_str());
    } else if (tag == "EDGE_WEIGHT_TYPE") {
      if (value != "EUC_2D") {
        delete t;
        return tsplib_fail(ACO_ERR_FORMAT, "invalid edge weight type: " + value);
      }
    } else if (tag == "NODE_COORD_SECTION") {
      if (nodes < 1 || nodes >= (1L << 21)) {
        delete t;
        return tsplib_fail(ACO_ERR_FORMAT, "NODE_COORD_SECTION without a valid DIMENSION");
      }
      t->x.assign((size_t)nodes, 0.0f);
      t->y.assign((size_t)nodes, 0.0f);
      for (long i = 0; i < nodes; i++) {
        if (!in.good()) {
          delete t;
          return tsplib_fail(ACO_ERR_FORMAT, "file ends inside NODE_COORD_SECTION");
        }
        std::getline(in, line);
        strip_trailing_unprintable(line);
        if (line == "EOF") {
          delete t;
          return tsplib_fail(ACO_ERR_FORMAT, "EOF inside NODE_COORD_SECTION");
        }
        long id = 0;
        if (sscanf(line.c_str(), "%ld %f %f", &id, &t->x[(size_t)i], &t->y[(size_t)i]) != 3) {
          delete t;
          return tsplib_fail(ACO_ERR_FORMAT, "unreadable coordinate line: " + line);
        }
      }
      have_coords = true;
    }
    if (line == "EOF") break;
  }
  if (!have_coords) {
    delete t;
    return tsplib_fail(ACO_ERR_FORMAT, "no NODE_COORD_SECTION");
  }
  *out = t;
  return ACO_OK;
}

int32_t aco_tsplib_num_nodes(const aco_tsplib *t) { return t ? (int32_t)t->x.size() : 0; }

const char *aco_tsplib_name(const aco_tsplib *t) { return t ? t->name.c_str() : ""; }

const float *aco_tsplib_xcoords(const aco_tsplib *t) { return t ? t->x.data() : nullptr; }

const float *aco_tsplib_ycoords(const aco_tsplib *t) { return t ? t->y.data() : nullptr; }

const char *aco_tsplib_last_error(void) { return g_tsplib_error.c_str(); }

void aco_tsplib_destroy(aco_tsplib *t) { delete t; }

}  // extern "C"

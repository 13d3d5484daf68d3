// Verbosity-filtered messages and the fatal-error exit of the legacy API.
#include "log.h"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace ommp {

namespace {
int g_level = kVerbLow;  // OMMP_VERBOSE_DEFAULT
FILE *g_out = nullptr;   // nullptr = stdout
std::mutex g_mu;

void emit(const char *tag, const char *text) {
  char pre[16];
  char br[32];
  snprintf(br, sizeof br, "[%s]", tag);
  snprintf(pre, sizeof pre, "%12.12s", br);
  FILE *f = g_out ? g_out : stdout;
  fprintf(f, "[OMMP]%s %s\n", pre, text);
  fflush(f);
}
}  // namespace

void log_set_level(int v) { g_level = v < 0 ? 0 : (v > 3 ? 3 : v); }
int log_level() { return g_level; }

void log_set_file(const char *path) {
  std::lock_guard<std::mutex> lk(g_mu);
  FILE *f = fopen(path, "w");
  if (!f) {
    emit("stop", "Error while opening output input file");
    emit("stop", "Unrecoverable error in openMMPol library. Exiting.");
    exit(1);
  }
  char msg[4200];
  snprintf(msg, sizeof msg, "Switching output from stdout to %s.", path);
  if (g_level >= kVerbLow) emit("warning", msg);
  if (g_out) fclose(g_out);
  g_out = f;
}

void log_close_file() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_out) {
    fclose(g_out);
    g_out = nullptr;
  }
}

void log_msg(int level, const char *tag, const char *fmt, ...) {
  if (level > g_level) return;
  char text[4096];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(text, sizeof text, fmt, ap);
  va_end(ap);
  if (!tag) tag = level == kVerbLow ? "warning" : (level == kVerbHigh ? "info" : "debug");
  std::lock_guard<std::mutex> lk(g_mu);
  emit(tag, text);
}

void log_fatal(const char *msg) {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    // like the reference, the "stop" lines are level-LOW messages
    if (g_level >= kVerbLow) {
      emit("stop", msg);
      emit("stop", "Unrecoverable error in openMMPol library. Exiting.");
    }
    if (g_out) fclose(g_out);
    g_out = nullptr;
  }
  exit(1);
}

}  // namespace ommp

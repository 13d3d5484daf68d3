// Message channel with the reference's verbosity levels and line format
// ("[OMMP]" + right-aligned "[tag]" in 12 columns + text; src/mod_io.F90:110-153).
#pragma once

namespace ommp {

constexpr int kVerbNone = 0, kVerbLow = 1, kVerbHigh = 2, kVerbDebug = 3;

void log_set_level(int v);
int log_level();
void log_set_file(const char *path);
void log_close_file();
// tag == nullptr picks the reference's default tag for the level
void log_msg(int level, const char *tag, const char *fmt, ...) __attribute__((format(printf, 3, 4)));
// prints the message with the "stop" tag and terminates the process (exit 1)
[[noreturn]] void log_fatal(const char *msg);

}  // namespace ommp

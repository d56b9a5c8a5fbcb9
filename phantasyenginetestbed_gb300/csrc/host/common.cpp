#include "common.hpp"

namespace phe_gb300 {

static thread_local std::string g_lastError;

phe_status fail(phe_status status, const char* fmt, ...)
{
	char buf[1024];
	va_list ap;
	va_start(ap, fmt);
	std::vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_lastError = buf;
	return status;
}

void clear_error() { g_lastError.clear(); }

} // namespace phe_gb300

extern "C" const char* phe_last_error(void) { return phe_gb300::g_lastError.c_str(); }
extern "C" int phe_version(void) { return 100; }

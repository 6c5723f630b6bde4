// Stub: logging is dropped in the known-answer bridge.
#pragma once
#define KALYPSSO_INFO(...) ((void)0)
#define KALYPSSO_ERROR(...) ((void)0)
#define KALYPSSO_WARNING(...) ((void)0)

// Forced-include header for the timed reference checker build: the reference
// defines ENABLE_METRICS unconditionally (core/CrossRT.h:31), which adds racy
// per-node counters to every traversal step.  The timed build includes
// CrossRT.h first and then drops the macro, as the reference's own renderers
// would see it with metrics switched off.
#pragma once
#undef ENABLE_METRICS

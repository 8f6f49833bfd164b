// matplot.h -- the samples' spike output (spike_output_stream, pause) for this engine's population
// handles, so the reference's sample programs compile against include/spice/snn.h plus this
// directory.  Prints the JSON raster of samples/matplot.cpp:96-134 to stdout: per step, the spikes
// of the streamed populations in stream order, each population's indices offset by the sizes of
// the populations streamed before it; skip_steps_without_spikes leaves out populations without
// spikes in that step.  The animated matplot++ window of the reference is not built (no graphics
// stack); pause() does nothing.
#pragma once

#include <cstdio>
#include <string>

#include "spice/snn.h"

inline void pause(double) {}

class spike_output_stream {
public:
	explicit spike_output_stream(std::string const& model_name, bool const skip_steps_without_spikes = false) :
	_skip(skip_steps_without_spikes) {
		std::printf("{\n\t\"name\": \"%s\",\n\t\"spikes\": [\n", model_name.c_str());
	}
	~spike_output_stream() { std::printf("\n\t]\n}\n"); }
	spike_output_stream(spike_output_stream const&)            = delete;
	spike_output_stream& operator=(spike_output_stream const&) = delete;

	template <class Neur>
	spike_output_stream& operator<<(spice::neuron_population<Neur> const* pop) {
		auto const s = pop->spikes(0);
		if (!_skip || !s.empty()) {
			for (auto x : s) {
				std::printf("%s%lld", _delim, (long long)x + (long long)_offset);
				_delim = ",";
			}
			_offset += pop->size();
		}
		return *this;
	}
	spike_output_stream& operator<<(char const c) {
		if (c == '\n') {
			if (_offset > 0) {
				_delim = ",\n\t\t[";
				std::printf("]");
			}
			_offset = 0;
		}
		return *this;
	}

private:
	bool _skip;
	long long _offset  = 0;
	char const* _delim = "\t\t[";
};

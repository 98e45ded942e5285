// Live stream ingest (host only): LIVESIM frame headers, TCP framing and the per-channel
// SIM sequence detection of the reference's live mode.
//
// Header: transport/ImageWrapper.java:418-478 (writeHeader / parseHeader; little endian).
// Framing: transport/ImageReceiver.java:122-164 (header, then width*height*bpp payload
// bytes; a broken header ends the connection).
// Sequence detection: livemode/SimSequenceExtractor.java. The reference runs one blocking
// thread per channel (PerChannelBuffer.run, :397-477) that pulls frames in sequence-number
// order through a 20-slot sort buffer (getSorted / sortFromQueue / setSeqNr, :262-344),
// searches a sync frame, then copies SyncFrameFreq sequences of nrDirs*nrPhases frames. Here
// the same algorithm is an explicit state machine per channel, advanced by every push: a
// pull that would block in the reference returns "needs input" instead, with exactly the
// state the blocked thread would hold, so the sequences are those the reference forms from
// the same per-channel frame order. JoinedChannelBuffer (:185-204) becomes pop(): one
// sequence of every channel, in channel order.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <limits>
#include <map>
#include <mutex>
#include <vector>

#include "fairsim_gb300.h"

namespace fsim {
void set_error(const char* fmt, ...);
}
using fsim::set_error;

namespace {

template <class T>
T rd(const uint8_t* b, int off) {  // little-endian load of any width, byte by byte
  uint64_t v = 0;
  for (int i = (int)sizeof(T) - 1; i >= 0; i--) v = (v << 8) | b[off + i];
  T r;
  std::memcpy(&r, &v, sizeof(T));
  return r;
}
template <class T>
void wr(uint8_t* b, int off, T val) {
  uint64_t v = 0;
  std::memcpy(&v, &val, sizeof(T));
  for (int i = 0; i < (int)sizeof(T); i++) b[off + i] = (uint8_t)(v >> (8 * i));
}

int parse(const uint8_t* b, int max_w, int max_h, fsim_livesim_header* h) {
  h->seq_nr = rd<int64_t>(b, 0);
  h->payload_offset = rd<int32_t>(b, 8);
  h->payload_len = rd<int32_t>(b, 12);
  h->version = rd<int8_t>(b, 16);
  h->bytes_per_pixel = rd<int8_t>(b, 17);
  h->width = rd<int16_t>(b, 32);
  h->height = rd<int16_t>(b, 34);
  h->pos_a = rd<int16_t>(b, 36);
  h->pos_b = rd<int16_t>(b, 38);
  h->pos0 = rd<int16_t>(b, 40);
  h->pos1 = rd<int16_t>(b, 42);
  h->pos2 = rd<int32_t>(b, 44);
  h->time_camera = rd<int64_t>(b, 48);
  h->time_capture = rd<int64_t>(b, 56);
  h->time_record = rd<int64_t>(b, 64);
  // the checks of ImageWrapper.parseHeader, in its order (a width or height that reads
  // negative as int16 is rejected too: the reference would fail allocating the frame)
  if (h->width > max_w || h->height > max_h || h->width < 0 || h->height < 0) {
    set_error("broken header: image too large, is/max, w: %d,%d, h: %d,%d", h->width, max_w, h->height, max_h);
    return FSIM_EINVAL;
  }
  if ((int64_t)h->payload_len != (int64_t)h->width * h->height) {
    set_error("broken header: width x height != len");
    return FSIM_EINVAL;
  }
  if (h->bytes_per_pixel != 1 && h->bytes_per_pixel != 2) {
    set_error("broken header: bpp neither 1 nor 2");
    return FSIM_EINVAL;
  }
  if (h->version != 1) {
    set_error("broken header: unsupported version");
    return FSIM_EINVAL;
  }
  return FSIM_OK;
}

struct Frame {
  int64_t seq = 0;
  int64_t t_cam = 0;
  std::vector<uint16_t> px;
};

// MTool.avr_ushort (linalg/MTool.java:68-76): mean of the unsigned values, in double
double avr_ushort(const std::vector<uint16_t>& p) {
  double r = 0;
  for (uint16_t v : p) r += v;
  return r / (double)p.size();
}

struct Channel {
  int number = 0;
  std::deque<Frame> raw;             // rawImgs (bounded)
  std::map<int64_t, Frame> sortbuf;  // SortBuffer (TreeMap, 20 slots)
  int64_t seqNr = 0;
  bool refill = true;  // setSeqNr pending (it runs when the thread starts)
  enum Phase { SEARCH, SKIP, COPY } phase = SEARCH;
  int64_t lastTs = 0, curTs = 0;
  int counter = 0, k = 0, i = 0;
  using Seq = std::vector<std::vector<uint16_t>>;  // the frames of one SIM sequence
  Seq cur;                                    // the sequence being collected
  std::deque<Seq> sims;                       // simSeq (bounded)
  std::deque<int64_t> sim_first;
  int64_t cur_first = 0;
  uint64_t missed_raw = 0, missed_sim = 0, syncs = 0, resyncs = 0, dups = 0;
};

}  // namespace

struct fsim_seqx {
  fsim_seqx_config cfg{};
  std::vector<Channel> ch;
  size_t frame_px = 0;
  int raw_cap = 0, sim_cap = 0;
  static constexpr int SORT_SLOTS = 20;     // SortBuffer(20)
  static constexpr int64_t SYNCJITTER = 50;  // PerChannelBuffer.SYNCJITTER
  uint64_t frames = 0, bytes = 0, unknown = 0, sequences = 0;
  // stream framing (fsim_seqx_feed): the partial frame at the end of the last piece
  std::vector<uint8_t> pend;
  bool closed = false;
  std::mutex mu;
  // recycled frame buffers: large allocations are otherwise mapped and faulted in anew for
  // every frame
  std::vector<std::vector<uint16_t>> pool_frame;

  std::vector<uint16_t> take(std::vector<std::vector<uint16_t>>& pool, size_t n) {
    std::vector<uint16_t> v;
    if (!pool.empty()) {
      v = std::move(pool.back());
      pool.pop_back();
    }
    v.resize(n);
    return v;
  }
  void give(std::vector<std::vector<uint16_t>>& pool, std::vector<uint16_t>&& v) {
    if (pool.size() < 256 && v.capacity()) pool.push_back(std::move(v));
  }

  int channel_of(int pos1) const {
    for (int c = 0; c < cfg.n_channels; c++)
      if (cfg.channel_numbers[c] == pos1) return c;
    return -1;
  }

  // SortBuffer.add: a second frame with a buffered sequence number is an error in the
  // reference (fatal there); here it is counted and the newer frame dropped
  void sort_add(Channel& c, Frame&& f) {
    auto it = c.sortbuf.find(f.seq);
    if (it != c.sortbuf.end()) {
      c.dups++;
      give(pool_frame, std::move(f.px));
      return;
    }
    c.sortbuf.emplace(f.seq, std::move(f));
  }

  // setSeqNr (:312-338): fill the sort buffer with raws_per_recon frames from the queue
  // and restart at the smallest sequence number among them. false: needs more frames.
  bool do_refill(Channel& c) {
    while ((int)c.sortbuf.size() < cfg.raws_per_recon) {
      if (c.raw.empty()) return false;
      Frame f = std::move(c.raw.front());
      c.raw.pop_front();
      if (f.seq < c.seqNr) c.seqNr = f.seq;
      sort_add(c, std::move(f));
    }
    c.refill = false;
    return true;
  }

  // getSorted / sortFromQueue (:262-298): the next frame in sequence-number order.
  // false: the reference's thread would block here for a frame (state kept).
  bool get_sorted(Channel& c, Frame& out) {
    for (;;) {
      if (c.refill && !do_refill(c)) return false;
      if (!c.sortbuf.empty()) {
        auto it = c.sortbuf.find(c.seqNr);
        if (it != c.sortbuf.end()) {
          out = std::move(it->second);
          c.sortbuf.erase(it);
          c.seqNr++;
          return true;
        }
      }
      if (c.raw.empty()) return false;
      Frame f = std::move(c.raw.front());
      c.raw.pop_front();
      if (f.seq == c.seqNr) {
        c.seqNr++;
        out = std::move(f);
        return true;
      }
      if ((int)c.sortbuf.size() < SORT_SLOTS) {
        sort_add(c, std::move(f));
        continue;
      }
      // BufferOverflowException: this frame is lost, the buffer re-sorted from the queue
      c.seqNr++;
      c.resyncs++;
      c.sortbuf.clear();
      c.seqNr = std::numeric_limits<int64_t>::max();
      c.refill = true;
    }
  }

  void emit(Channel& c) {
    if ((int)c.sims.size() < sim_cap) {
      c.sims.push_back(std::move(c.cur));
      c.sim_first.push_back(c.cur_first);
    } else {
      c.missed_sim++;
      for (auto& v : c.cur) give(pool_frame, std::move(v));
    }
    c.cur.clear();
  }

  // PerChannelBuffer.run (:397-477) as a state machine, run until it needs a frame
  void step(Channel& c) {
    const int nraw = cfg.raws_per_recon;
    Frame f;
    for (;;) {
      if (c.phase == Channel::SEARCH) {
        if (!get_sorted(c, f)) return;
        c.curTs = f.t_cam;
        if (cfg.sync_mode == 0) {
          // camera with time stamps: the first frame after a gap opens the sequence
          if (c.curTs - c.lastTs > cfg.sync_frame_delay) {
            if ((int)c.sortbuf.size() < SORT_SLOTS) {
              sort_add(c, std::move(f));
              c.seqNr--;
            }
            c.syncs++;
            c.phase = Channel::COPY;
            c.k = c.i = 0;
            continue;
          }
        } else {
          // precise time stamps: the frame after a gap of delay +- 50 us is the sync frame
          if (std::llabs(c.curTs - c.lastTs - cfg.sync_frame_delay) < SYNCJITTER) {
            c.syncs++;
            c.phase = Channel::COPY;
            c.k = c.i = 0;
            continue;
          }
          // no time stamps: a bright frame, and the frame after it is skipped
          if (avr_ushort(f.px) > (double)cfg.sync_frame_avr) {
            c.syncs++;
            c.phase = Channel::SKIP;
            continue;
          }
        }
        c.lastTs = c.curTs;
        if (++c.counter >= nraw * cfg.sync_frame_freq) c.counter = 0;  // "No sync frame found"
        give(pool_frame, std::move(f.px));
      } else if (c.phase == Channel::SKIP) {
        if (!get_sorted(c, f)) return;
        give(pool_frame, std::move(f.px));
        c.phase = Channel::COPY;
        c.k = c.i = 0;
      } else {
        if (!get_sorted(c, f)) return;
        if (c.i == 0) {
          c.cur.clear();
          c.cur.reserve(nraw);
          c.cur_first = f.seq;
        }
        c.cur.push_back(std::move(f.px));  // the frame's buffer joins the sequence
        c.curTs = f.t_cam;
        c.lastTs = c.curTs;
        if (++c.i == nraw) {
          emit(c);
          c.i = 0;
          if (++c.k == cfg.sync_frame_freq) {
            c.phase = Channel::SEARCH;
            c.counter = 0;
          }
        }
      }
    }
  }

  int push_frame(const uint8_t* b, size_t n) {
    fsim_livesim_header h;
    int rc = parse(b, cfg.width, cfg.height, &h);
    if (rc) return rc;
    const size_t payload = (size_t)h.width * h.height * h.bytes_per_pixel;
    if (n < FSIM_LIVESIM_HEADER_BYTES + payload) {
      set_error("frame: %zu bytes, header says %zu", n, FSIM_LIVESIM_HEADER_BYTES + payload);
      return FSIM_EINVAL;
    }
    frames++;
    const int ci = channel_of(h.pos1);
    if (ci < 0) {  // ImageSorter: "received data packet w/o channel"
      unknown++;
      set_error("frame %lld: no channel %d", (long long)h.seq_nr, h.pos1);
      return FSIM_ENOTFOUND;
    }
    if ((size_t)h.width * h.height != frame_px) {
      set_error("frame %lld: %d x %d, the channel's frames are %d x %d", (long long)h.seq_nr, h.width, h.height,
                cfg.width, cfg.height);
      return FSIM_EINVAL;
    }
    Channel& c = ch[ci];
    if ((int)c.raw.size() >= raw_cap) {  // PerChannelBuffer.pushImg: offer fails
      c.missed_raw++;
      return FSIM_OK;
    }
    Frame f;
    f.seq = h.seq_nr;
    f.t_cam = h.time_camera;
    f.px = take(pool_frame, frame_px);
    const uint8_t* p = b + FSIM_LIVESIM_HEADER_BYTES;
    if (h.bytes_per_pixel == 2) {
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
      std::memcpy(f.px.data(), p, frame_px * sizeof(uint16_t));  // the wire order is the host's
#else
      for (size_t i = 0; i < frame_px; i++) f.px[i] = (uint16_t)(p[2 * i] | (p[2 * i + 1] << 8));
#endif
    } else {
      // ImageWrapper.getPixels: ret[i] = buffer[i + HEADERSIZE], a signed Java byte
      for (size_t i = 0; i < frame_px; i++) f.px[i] = (uint16_t)(int16_t)(int8_t)p[i];
    }
    c.raw.push_back(std::move(f));
    step(c);
    return FSIM_OK;
  }

  void reset() {
    for (auto& c : ch) {
      const int num = c.number;
      c = Channel();
      c.number = num;
      c.seqNr = std::numeric_limits<int64_t>::max();
    }
    pend.clear();
    closed = false;
  }
};

extern "C" {

int fsim_livesim_parse(const void* header_bytes, int max_width, int max_height, fsim_livesim_header* out) {
  if (!header_bytes || !out) {
    set_error("livesim_parse: null argument");
    return FSIM_EINVAL;
  }
  return parse(static_cast<const uint8_t*>(header_bytes), max_width, max_height, out);
}

int fsim_livesim_write(const fsim_livesim_header* h, void* header_bytes) {
  if (!h || !header_bytes) {
    set_error("livesim_write: null argument");
    return FSIM_EINVAL;
  }
  uint8_t* b = static_cast<uint8_t*>(header_bytes);
  std::memset(b, 0, FSIM_LIVESIM_HEADER_BYTES);
  wr<int64_t>(b, 0, h->seq_nr);
  wr<int32_t>(b, 12, h->width * h->height);
  wr<int8_t>(b, 16, 1);
  wr<int8_t>(b, 17, (int8_t)h->bytes_per_pixel);
  wr<int16_t>(b, 32, (int16_t)h->width);
  wr<int16_t>(b, 34, (int16_t)h->height);
  wr<int16_t>(b, 36, (int16_t)h->pos_a);
  wr<int16_t>(b, 38, (int16_t)h->pos_b);
  wr<int16_t>(b, 40, (int16_t)h->pos0);
  wr<int16_t>(b, 42, (int16_t)h->pos1);
  wr<int32_t>(b, 44, h->pos2);
  wr<int64_t>(b, 48, h->time_camera);
  wr<int64_t>(b, 56, h->time_capture);
  wr<int64_t>(b, 64, h->time_record);
  return FSIM_OK;
}

int fsim_seqx_create(fsim_seqx** out, const fsim_seqx_config* cfg) {
  if (!out || !cfg) {
    set_error("seqx_create: null argument");
    return FSIM_EINVAL;
  }
  *out = nullptr;
  if (cfg->n_channels < 1 || cfg->n_channels > FSIM_MAX_CHANNELS || cfg->raws_per_recon < 1 ||
      cfg->raws_per_recon > 20 || cfg->width < 1 || cfg->height < 1 || cfg->width > 32767 ||
      cfg->height > 32767 || (cfg->sync_mode != 0 && cfg->sync_mode != 1) || cfg->sync_frame_freq < 1 ||
      cfg->raw_queue < 0 || cfg->sim_queue < 0) {
    set_error("seqx_create: bad configuration (channels 1..%d, raws per recon 1..20, sync mode 0/1, "
              "sync frequency >= 1)", FSIM_MAX_CHANNELS);
    return FSIM_EINVAL;
  }
  for (int a = 0; a < cfg->n_channels; a++)
    for (int b = a + 1; b < cfg->n_channels; b++)
      if (cfg->channel_numbers[a] == cfg->channel_numbers[b]) {
        set_error("seqx_create: channel number %d given twice", cfg->channel_numbers[a]);
        return FSIM_EINVAL;
      }
  fsim_seqx* s = new (std::nothrow) fsim_seqx();
  if (!s) {
    set_error("seqx_create: out of memory");
    return FSIM_EOOM;
  }
  s->cfg = *cfg;
  s->frame_px = (size_t)cfg->width * cfg->height;
  const int q = cfg->raws_per_recon * cfg->raws_per_recon * 10;  // PerChannelBuffer queue size
  s->raw_cap = cfg->raw_queue ? cfg->raw_queue : q;
  s->sim_cap = cfg->sim_queue ? cfg->sim_queue : q;
  s->ch.resize(cfg->n_channels);
  for (int c = 0; c < cfg->n_channels; c++) s->ch[c].number = cfg->channel_numbers[c];
  s->reset();
  *out = s;
  return FSIM_OK;
}

int fsim_seqx_push(fsim_seqx* s, const void* frame, size_t bytes) {
  if (!s || !frame || bytes < FSIM_LIVESIM_HEADER_BYTES) {
    set_error("seqx_push: null argument or frame shorter than its header");
    return FSIM_EINVAL;
  }
  std::lock_guard<std::mutex> g(s->mu);
  s->bytes += bytes;
  return s->push_frame(static_cast<const uint8_t*>(frame), bytes);
}

int fsim_seqx_feed(fsim_seqx* s, const void* bytes, size_t n) {
  if (!s || (!bytes && n)) {
    set_error("seqx_feed: null argument");
    return FSIM_EINVAL;
  }
  std::lock_guard<std::mutex> g(s->mu);
  if (s->closed) {
    set_error("seqx_feed: the stream was closed by a broken header (fsim_seqx_reset reopens it)");
    return FSIM_EINVAL;
  }
  s->bytes += n;
  const uint8_t* b = static_cast<const uint8_t*>(bytes);
  int rc = FSIM_OK;
  auto frame_len = [&](const uint8_t* hdr, size_t* len) {
    fsim_livesim_header h;
    int prc = parse(hdr, s->cfg.width, s->cfg.height, &h);
    if (prc) {  // the reference's receiving thread ends: the connection is closed
      s->closed = true;
      s->pend.clear();
      return prc;
    }
    *len = FSIM_LIVESIM_HEADER_BYTES + (size_t)h.width * h.height * h.bytes_per_pixel;
    return FSIM_OK;
  };
  // complete the frame left partial by the previous piece
  if (!s->pend.empty()) {
    if (s->pend.size() < FSIM_LIVESIM_HEADER_BYTES) {
      const size_t k = std::min(n, FSIM_LIVESIM_HEADER_BYTES - s->pend.size());
      s->pend.insert(s->pend.end(), b, b + k);
      b += k;
      n -= k;
      if (s->pend.size() < FSIM_LIVESIM_HEADER_BYTES) return FSIM_OK;
    }
    size_t len = 0;
    int prc = frame_len(s->pend.data(), &len);
    if (prc) return prc;
    const size_t k = std::min(n, len - s->pend.size());
    s->pend.insert(s->pend.end(), b, b + k);
    b += k;
    n -= k;
    if (s->pend.size() < len) return FSIM_OK;
    if (s->push_frame(s->pend.data(), len) == FSIM_EINVAL) rc = FSIM_EINVAL;
    s->pend.clear();
  }
  // whole frames straight from this piece, then keep its tail
  while (n >= FSIM_LIVESIM_HEADER_BYTES) {
    size_t len = 0;
    int prc = frame_len(b, &len);
    if (prc) return prc;
    if (n < len) break;
    if (s->push_frame(b, len) == FSIM_EINVAL) rc = FSIM_EINVAL;  // a frame of another size: reported
    b += len;
    n -= len;
  }
  s->pend.assign(b, b + n);
  return rc;
}

int fsim_seqx_pop(fsim_seqx* s, uint16_t* out, int64_t* first_seq) {
  if (!s || !out) {
    set_error("seqx_pop: null argument");
    return FSIM_EINVAL;
  }
  std::lock_guard<std::mutex> g(s->mu);
  for (auto& c : s->ch)
    if (c.sims.empty()) return FSIM_ENOTFOUND;
  const size_t per = (size_t)s->cfg.raws_per_recon * s->frame_px;
  for (size_t c = 0; c < s->ch.size(); c++) {
    Channel& ch = s->ch[c];
    auto& seq = ch.sims.front();
    for (size_t i = 0; i < seq.size(); i++) {
      std::memcpy(out + c * per + i * s->frame_px, seq[i].data(), s->frame_px * sizeof(uint16_t));
      s->give(s->pool_frame, std::move(seq[i]));
    }
    if (first_seq) first_seq[c] = ch.sim_first.front();
    ch.sims.pop_front();
    ch.sim_first.pop_front();
  }
  s->sequences++;
  return FSIM_OK;
}

int fsim_seqx_stats_get(const fsim_seqx* s, fsim_seqx_stats* out) {
  if (!s || !out) {
    set_error("seqx_stats: null argument");
    return FSIM_EINVAL;
  }
  fsim_seqx* m = const_cast<fsim_seqx*>(s);
  std::lock_guard<std::mutex> g(m->mu);
  std::memset(out, 0, sizeof(*out));
  out->frames = s->frames;
  out->bytes = s->bytes;
  out->unknown_channel = s->unknown;
  out->sequences = s->sequences;
  for (size_t c = 0; c < s->ch.size(); c++) {
    out->missed_raw[c] = s->ch[c].missed_raw;
    out->missed_sim[c] = s->ch[c].missed_sim;
    out->sync_frames[c] = s->ch[c].syncs;
    out->resyncs[c] = s->ch[c].resyncs;
    out->duplicates[c] = s->ch[c].dups;
  }
  return FSIM_OK;
}

int fsim_seqx_reset(fsim_seqx* s) {
  if (!s) {
    set_error("seqx_reset: null argument");
    return FSIM_EINVAL;
  }
  std::lock_guard<std::mutex> g(s->mu);
  s->reset();
  return FSIM_OK;
}

int fsim_seqx_destroy(fsim_seqx* s) {
  delete s;
  return FSIM_OK;
}

}  // extern "C"
